// C ABI of libheatflow_gb300 (include/heatflow_gb300.h): context set-up, state transfer and the
// host side of the step loop.  Host arithmetic here is the reference's set-up arithmetic
// (cell lengths, volumes, heated volume, Neumann power densities) and is compiled without FMA
// contraction so it rounds as the reference does.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "hf_ctx.cuh"

#define HF_FILE_ID 1   // index-check sites of the checked build: 100000 * file + line

namespace hf {
cudaError_t launch_props(Ctx& c, const double* rho, const double* hc, const double* tau,
                         const double* em);
}

using namespace hf;

struct hf_ctx {
  Ctx c;
};

static thread_local std::string g_err;

static int set_err(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

namespace hf {
void set_last_error(const std::string& msg) { g_err = msg; }
}

#define CU(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return set_err(HF_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));      \
  } while (0)

extern "C" {

int hf_abi_version(void) { return HF_ABI_VERSION; }

const char* hf_strerror(int code) {
  switch (code) {
    case HF_OK: return "ok";
    case HF_EARG: return "invalid argument";
    case HF_ECUDA: return "CUDA error";
    case HF_ENOMEM: return "device allocation failed";
    case HF_ESTATE: return "call order error";
    case HF_EDEVICE: return "device-side check failed";
    case HF_ENAN_B: return "fatal error: NAN in B vector";
    case HF_ENAN_Q: return "fatal error: NAN in Q vector";
    case HF_ENAN_QDENS: return "fatal error: NAN in Qdens vector";
    case HF_ENAN_SCAT: return "fatal error: NAN in S_CAT vector";
    case HF_ENAN_S: return "fatal error: NAN in S vector";
    case HF_ENAN_X: return "fatal error: NAN in x tempurature vector";
    default: return "unknown status";
  }
}

const char* hf_last_error(void) { return g_err.c_str(); }

void hf_default_opts(hf_solver_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->precision = HF_PREC_FP64;
  o->criterion = HF_STOP_RECURSIVE;
  o->tol = 1.0e-32;        // mod_evolve.f90:143
  o->itmax = 50000;        // mod_evolve.f90:144
  o->inner_tol = 1.0e-4;
  o->inner_itmax = 200;
  o->max_refine = 20;
  o->check_every = 2;
  o->use_graph = 0;
  o->task_depth = 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
namespace {

template <typename T>
int dalloc(Ctx& c, T** p, size_t count) {
  void* q = nullptr;
  size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_err(HF_ENOMEM, std::string("cudaMalloc ") + std::to_string(bytes) + " bytes: " +
                                  cudaGetErrorString(e));
  }
  c.allocs.push_back(q);
  *p = static_cast<T*>(q);
  return HF_OK;
}

void drop_graph(Ctx& c) {
  if (c.graph_exec) cudaGraphExecDestroy(c.graph_exec);
  if (c.graph) cudaGraphDestroy(c.graph);
  c.graph_exec = nullptr;
  c.graph = nullptr;
  if (c.loop_exec) cudaGraphExecDestroy(c.loop_exec);
  if (c.loop_graph) cudaGraphDestroy(c.loop_graph);
  c.loop_exec = nullptr;
  c.loop_graph = nullptr;
  for (int j = 0; j < 2; ++j) {
    if (c.post_exec[j]) cudaGraphExecDestroy(c.post_exec[j]);
    if (c.post_graph[j]) cudaGraphDestroy(c.post_graph[j]);
    c.post_exec[j] = nullptr;
    c.post_graph[j] = nullptr;
  }
}

void free_all(Ctx& c) {
  if (c.stream) cudaStreamSynchronize(c.stream);   // queued host-buffer steps may still run
  drop_graph(c);
  if (c.out_stream) cudaStreamSynchronize(c.out_stream);
  if (c.ev_gathered) cudaEventDestroy(c.ev_gathered);
  c.ev_gathered = nullptr;
  for (auto& o : c.outs) {
    if (o.done) cudaEventDestroy(o.done);
    o.done = nullptr;
    for (auto& e : o.chunk) {
      if (e) cudaEventDestroy(e);
      e = nullptr;
    }
    o.ptr = nullptr;
  }
  for (auto& e : c.stage_x_free) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  for (auto& st : c.stage) {
    for (cudaEvent_t* e : {&st.in_pp, &st.free}) {
      if (*e) cudaEventDestroy(*e);
      *e = nullptr;
    }
    for (auto& e : st.in_chunk) {
      if (e) cudaEventDestroy(e);
      e = nullptr;
    }
  }
  if (c.copy_stream) cudaStreamSynchronize(c.copy_stream);
  for (auto& sl : c.sub) {
    if (sl.dev) cudaFree(sl.dev);
    if (sl.gathered) cudaEventDestroy(sl.gathered);
    if (sl.copied) cudaEventDestroy(sl.copied);
    sl = Ctx::SubSlot{};
  }
  if (c.copy_stream) cudaStreamDestroy(c.copy_stream);
  c.copy_stream = nullptr;
  if (c.out_stream) cudaStreamDestroy(c.out_stream);
  c.out_stream = nullptr;
  for (void* p : c.allocs) cudaFree(p);
  c.allocs.clear();
  if (c.h_scal) cudaFreeHost(c.h_scal);
  c.h_scal = nullptr;
  if (c.own_stream && c.stream) cudaStreamDestroy(c.stream);
  c.stream = nullptr;
}

DevOpts dev_opts(const hf_solver_opts& o) {
  DevOpts d{};
  d.precision = o.precision;
  d.criterion = o.criterion;
  d.tol = o.tol;
  d.itmax = o.itmax;
  d.inner_tol = o.inner_tol;
  d.inner_itmax = o.inner_itmax;
  d.max_refine = o.max_refine;
  return d;
}

int validate_opts(const hf_solver_opts& o) {
  if (o.precision != HF_PREC_FP64 && o.precision != HF_PREC_MIXED)
    return set_err(HF_EARG, "precision must be HF_PREC_FP64 or HF_PREC_MIXED");
  if (o.criterion != HF_STOP_RECURSIVE && o.criterion != HF_STOP_TRUE)
    return set_err(HF_EARG, "criterion must be HF_STOP_RECURSIVE or HF_STOP_TRUE");
  if (o.criterion == HF_STOP_RECURSIVE && o.precision != HF_PREC_FP64)
    return set_err(HF_EARG, "the reference's recursive criterion is defined for the FP64 path");
  if (!(o.tol >= 0.0) || o.itmax < 1 || o.inner_itmax < 1 || o.max_refine < 1 || o.check_every < 1)
    return set_err(HF_EARG, "tol >= 0, itmax, inner_itmax, max_refine, check_every >= 1");
  if (o.use_graph < 0 || o.use_graph > 3) return set_err(HF_EARG, "use_graph must be 0, 1, 2 or 3");
  if (o.task_depth != 0 && (o.task_depth < kMinTaskDepth || o.task_depth > 1024))
    return set_err(HF_EARG, "task_depth must be 0 (default) or 4..1024");
  return HF_OK;
}

// Calls that read or change a context's device state while host-buffer steps are queued
// (hf_step_host_async) are refused until hf_host_sync has collected them.
int refuse_queued(const Ctx& c) {
  return c.async_pending
             ? set_err(HF_ESTATE, "host-buffer steps are queued: call hf_host_sync first")
             : HF_OK;
}

int sync_scal(Ctx& c) {
  if (int r = refuse_queued(c)) return r;
  CU(cudaMemcpyAsync(c.h_scal, c.A.scal, sizeof(InstScal) * c.ninst, cudaMemcpyDeviceToHost,
                     c.stream));
  CU(cudaStreamSynchronize(c.stream));
  return HF_OK;
}

// Scalars written from the host mean state or scratch changed outside the step sequence (a restored
// snapshot, a timing run, a standalone solve, a new state): the stored products H T^n, H T^(n-1)
// are then not trusted, unless the caller restored them too (keep_hx).
int push_scal(Ctx& c, bool keep_hx = false) {
  if (!keep_hx)
    for (int64_t i = 0; i < c.ninst; ++i) c.h_scal[i].hx_ok = 0;
  CU(cudaMemcpyAsync(c.A.scal, c.h_scal, sizeof(InstScal) * c.ninst, cudaMemcpyHostToDevice,
                     c.stream));
  CU(cudaStreamSynchronize(c.stream));
  return HF_OK;
}

// First NaN code of an instance's status bits, in the reference's check order.
int status_code(int bits) {
  for (int k = 0; k <= HF_ENAN_X - HF_ENAN_B; ++k)
    if (bits & (1 << k)) return HF_ENAN_B + k;
  if (bits & kStatusRhsNan) return HF_ENAN_S;
  return HF_OK;
}

// A NaN in S was detected through ||S||^2: find which vector failed first, in the reference's
// check order (mod_evolve.f90:82-127), by re-running the failed step's RHS with per-vector tests.
int diagnose(Ctx& c) {
  bool any = false;
  for (int64_t i = 0; i < c.ninst; ++i) any |= (c.h_scal[i].status & kStatusRhsNan) != 0;
  if (!any) return HF_OK;
  CU(launch_rhs_diagnose(c));
  CU(launch_finalize(c, FIN_RHS_DIAG, nullptr, 0, 0));
  return sync_scal(c);
}

// Drive one step's solve after the RHS / initial residual kernels are queued.
int solve_loop(Ctx& c) {
  const bool fp32 = c.opts.precision == HF_PREC_MIXED;
  const int64_t per_solve = fp32 ? c.opts.inner_itmax : c.opts.itmax;
  const int64_t guard = (int64_t)(c.opts.max_refine + 3) * (per_solve / c.opts.check_every + 3);
  for (int64_t it = 0; it < guard; ++it) {
    int rc = sync_scal(c);
    if (rc) return rc;
    bool any_outer = false, any_inner = false;
    for (int64_t i = 0; i < c.ninst; ++i) {
      any_outer |= c.h_scal[i].outer_active != 0;
      any_inner |= c.h_scal[i].inner_active != 0;
    }
    if (!any_outer) return HF_OK;
    if (any_inner) {
      for (int k = 0; k < c.opts.check_every; ++k) CU(launch_inner_iteration(c, fp32 ? 1 : 0));
      c.launches += 5 * c.opts.check_every;
    } else {
      CU(launch_residual(c, 1));
      c.launches += 3;
    }
  }
  return set_err(HF_EDEVICE, "solve loop did not terminate within its bound");
}

int run_one_step(Ctx& c, int64_t itime) {
  CU(launch_step_begin(c, itime, 0));
  CU(launch_rhs(c));
  CU(launch_finalize(c, FIN_RHS, nullptr, 0, 0));
  CU(launch_residual(c, 0));
  c.launches += 5;
  int rc = solve_loop(c);
  if (rc) return rc;
  CU(launch_step_end(c));
  c.launches += 1;
  if (c.tempdep) {
    CU(launch_tempdep(c));
    c.launches += 4;
  }
  return HF_OK;
}

// Capture one step as a CUDA graph: the solve loop is a WHILE node whose body selects, through a
// SWITCH node, one inner CG iteration or one residual sweep; control kernels set the conditions
// from the per-instance phase flags, so a step runs without any host round trip.
int build_graph_cond(Ctx& c) {
  if (!c.d_ctrl) {
    int r = dalloc(c, &c.d_ctrl, 1);
    if (r) return r;
    CU(cudaMemset(c.d_ctrl, 0, sizeof(CtrlState)));
  }
  const bool fp32 = c.opts.precision == HF_PREC_MIXED;
  cudaStream_t cs = nullptr, cs2 = nullptr;
  CU(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  CU(cudaStreamCreateWithFlags(&cs2, cudaStreamNonBlocking));
  cudaStream_t saved = c.stream;
  cudaGraph_t g = nullptr;
  std::string err;
  auto chk = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && err.empty()) err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaSuccess;
  };
  do {
    if (!chk(cudaGraphCreate(&g, 0), "cudaGraphCreate")) break;
    cudaGraphConditionalHandle hw;
    if (!chk(cudaGraphConditionalHandleCreate(&hw, g, 0, cudaGraphCondAssignDefault), "handle(while)")) break;
    if (!chk(cudaStreamBeginCaptureToGraph(cs, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed), "capture")) break;
    c.stream = cs;
    chk(launch_graph_step_begin(c, c.d_ctrl, c.tempdep ? 10 : 6), "step begin");
    chk(launch_rhs(c), "rhs");
    chk(launch_finalize(c, FIN_RHS, c.d_ctrl, hw, 1), "rhs finalize");
    chk(launch_residual(c, 0, c.d_ctrl, hw, 1), "residual init");
    cudaStreamCaptureStatus st;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    chk(cudaStreamGetCaptureInfo(cs, &st, nullptr, &cg, &deps, nullptr, &nd), "capture info");
    cudaGraphNodeParams wp = {};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = hw;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode = nullptr;
    if (!chk(cudaGraphAddNode(&wnode, cg, deps, nullptr, nd, &wp), "while node")) { cudaStreamEndCapture(cs, &g); break; }
    cudaGraph_t body = wp.conditional.phGraph_out[0];
    chk(cudaStreamUpdateCaptureDependencies(cs, &wnode, nullptr, 1, cudaStreamSetCaptureDependencies), "deps");
    // loop body: select, switch, condition
    cudaGraphConditionalHandle hs;
    chk(cudaGraphConditionalHandleCreate(&hs, body, 2, cudaGraphCondAssignDefault), "handle(switch)");
    chk(cudaStreamBeginCaptureToGraph(cs2, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed), "capture body");
    c.stream = cs2;
    chk(launch_ctrl_select(c, c.d_ctrl, hs, hw), "select");
    cudaGraph_t cg2 = nullptr;
    const cudaGraphNode_t* deps2 = nullptr;
    size_t nd2 = 0;
    chk(cudaStreamGetCaptureInfo(cs2, &st, nullptr, &cg2, &deps2, nullptr, &nd2), "capture info body");
    cudaGraphNodeParams sp = {};
    sp.type = cudaGraphNodeTypeConditional;
    sp.conditional.handle = hs;
    sp.conditional.type = cudaGraphCondTypeSwitch;
    sp.conditional.size = 2;
    cudaGraphNode_t snode = nullptr;
    chk(cudaGraphAddNode(&snode, cg2, deps2, nullptr, nd2, &sp), "switch node");
    chk(cudaStreamUpdateCaptureDependencies(cs2, &snode, nullptr, 1, cudaStreamSetCaptureDependencies), "deps body");
    cudaGraph_t tmp = nullptr;
    chk(cudaStreamEndCapture(cs2, &tmp), "end body");
    if (err.empty()) {
      chk(cudaStreamBeginCaptureToGraph(cs2, sp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                        cudaStreamCaptureModeRelaxed), "capture cg");
      chk(launch_inner_iteration(c, fp32 ? 1 : 0, c.d_ctrl, hw, 1), "cg iteration");
      chk(cudaStreamEndCapture(cs2, &tmp), "end cg");
      chk(cudaStreamBeginCaptureToGraph(cs2, sp.conditional.phGraph_out[1], nullptr, nullptr, 0,
                                        cudaStreamCaptureModeRelaxed), "capture residual");
      chk(launch_residual(c, 1, c.d_ctrl, hw, 1), "residual");
      chk(cudaStreamEndCapture(cs2, &tmp), "end residual");
    }
    c.stream = cs;
    chk(launch_graph_step_end(c, c.d_ctrl, nullptr), "step end");
    if (c.tempdep) chk(launch_tempdep(c), "properties");
    cudaGraph_t outg = nullptr;
    chk(cudaStreamEndCapture(cs, &outg), "end capture");
    if (err.empty()) chk(cudaGraphInstantiate(&c.graph_exec, g, 0), "instantiate");
  } while (0);
  c.stream = saved;
  cudaStreamDestroy(cs);
  cudaStreamDestroy(cs2);
  if (!err.empty()) {
    if (c.graph_exec) cudaGraphExecDestroy(c.graph_exec);
    c.graph_exec = nullptr;
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return set_err(HF_ECUDA, "graph capture: " + err);
  }
  c.graph = g;
  return HF_OK;
}

// Capture one step with the persistent solve: step begin, RHS and its finalize, the cooperative
// solve kernel (zeroing its control block first), step end.  Five kernels per step.
int build_graph_persistent(Ctx& c) {
  if (!c.d_ctrl) {
    int r = dalloc(c, &c.d_ctrl, 1);
    if (r) return r;
    CU(cudaMemset(c.d_ctrl, 0, sizeof(CtrlState)));
  }
  if (solve_grid_blocks(c, c.opts.precision == HF_PREC_MIXED ? 1 : 0) < 1)
    return set_err(HF_ECUDA, "no co-resident grid for the persistent solve kernel");
  cudaStream_t cs = nullptr;
  CU(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaStream_t saved = c.stream;
  cudaGraph_t g = nullptr;
  std::string err;
  auto chk = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && err.empty()) err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaSuccess;
  };
  if (chk(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed), "capture")) {
    c.stream = cs;
    chk(launch_graph_step_begin(c, c.d_ctrl, c.tempdep ? 9 : 5), "step begin");
    chk(launch_rhs(c), "rhs");
    chk(launch_finalize(c, FIN_RHS, nullptr, 0, 0), "rhs finalize");
    chk(launch_solve(c), "persistent solve");
    chk(launch_graph_step_end(c, c.d_ctrl, c.d_sctl), "step end");
    if (c.tempdep) chk(launch_tempdep(c), "properties");
    chk(cudaStreamEndCapture(cs, &g), "end capture");
    if (err.empty()) chk(cudaGraphInstantiate(&c.graph_exec, g, 0), "instantiate");
  }
  c.stream = saved;
  cudaStreamDestroy(cs);
  if (!err.empty()) {
    if (c.graph_exec) cudaGraphExecDestroy(c.graph_exec);
    c.graph_exec = nullptr;
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return set_err(HF_ECUDA, "graph capture: " + err);
  }
  c.graph = g;
  return HF_OK;
}

// The whole time loop as one graph: a WHILE conditional node whose body is one step (step begin,
// RHS and its finalize, the persistent solve, step end).  k_graph_step_end sets the condition
// from the device step counter (CtrlState::itime < itime_end, and no failed solve), so a single
// launch runs any number of steps and always ends.  Built once per options; not every runtime
// accepts a cooperative kernel in a conditional body, and then hf_run launches the per-step graph
// back to back instead.
int build_loop_graph(Ctx& c) {
  if (c.loop_exec) return HF_OK;
  if (c.loop_unsupported) return HF_EARG;
  if (!c.d_ctrl) {
    int r = dalloc(c, &c.d_ctrl, 1);
    if (r) return r;
    CU(cudaMemset(c.d_ctrl, 0, sizeof(CtrlState)));
  }
  if (solve_grid_blocks(c, c.opts.precision == HF_PREC_MIXED ? 1 : 0) < 1)
    return set_err(HF_ECUDA, "no co-resident grid for the persistent solve kernel");
  cudaStream_t cs = nullptr;
  CU(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaStream_t saved = c.stream;
  cudaGraph_t g = nullptr;
  std::string err;
  auto chk = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && err.empty()) err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaSuccess;
  };
  do {
    if (!chk(cudaGraphCreate(&g, 0), "cudaGraphCreate")) break;
    cudaGraphConditionalHandle hl;
    if (!chk(cudaGraphConditionalHandleCreate(&hl, g, 1, cudaGraphCondAssignDefault), "handle")) break;
    cudaGraphNodeParams wp = {};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = hl;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode = nullptr;
    if (!chk(cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &wp), "while node")) break;
    cudaGraph_t body = wp.conditional.phGraph_out[0];
    if (!chk(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed),
             "capture body")) break;
    c.stream = cs;
    chk(launch_graph_step_begin(c, c.d_ctrl, c.tempdep ? 9 : 5), "step begin");
    chk(launch_rhs(c), "rhs");
    chk(launch_finalize(c, FIN_RHS, nullptr, 0, 0), "rhs finalize");
    chk(launch_solve(c), "persistent solve");
    chk(launch_graph_step_end(c, c.d_ctrl, c.d_sctl, hl, 1), "step end");
    if (c.tempdep) chk(launch_tempdep(c), "properties");
    cudaGraph_t tmp = nullptr;
    chk(cudaStreamEndCapture(cs, &tmp), "end capture");
    if (err.empty()) chk(cudaGraphInstantiate(&c.loop_exec, g, 0), "instantiate");
  } while (0);
  c.stream = saved;
  cudaStreamDestroy(cs);
  if (!err.empty()) {
    if (c.loop_exec) cudaGraphExecDestroy(c.loop_exec);
    c.loop_exec = nullptr;
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    c.loop_unsupported = true;
    return set_err(HF_ECUDA, "whole-loop graph: " + err);
  }
  c.loop_graph = g;
  return HF_OK;
}

int build_graph(Ctx& c) {
  if (c.graph_exec && c.graph_precision == c.opts.precision &&
      c.graph_criterion == c.opts.criterion && c.graph_mode == c.opts.use_graph)
    return HF_OK;
  drop_graph(c);
  const int rc = c.opts.use_graph == 2 ? build_graph_cond(c) : build_graph_persistent(c);
  if (rc) return rc;
  c.graph_precision = c.opts.precision;
  c.graph_criterion = c.opts.criterion;
  c.graph_mode = c.opts.use_graph;
  return HF_OK;
}

// The step after its RHS (RHS finalize, persistent solve, step end, property rebuild) as one
// graph, for steps whose RHS runs chunk by chunk behind the host upload (hf_step_host_async).
int build_post_graph(Ctx& c) {
  if (c.post_exec[0] && c.post_exec[1] && c.post_precision == c.opts.precision &&
      c.post_criterion == c.opts.criterion)
    return HF_OK;
  for (int j = 0; j < 2; ++j) {
    if (c.post_exec[j]) cudaGraphExecDestroy(c.post_exec[j]);
    if (c.post_graph[j]) cudaGraphDestroy(c.post_graph[j]);
    c.post_exec[j] = nullptr;
    c.post_graph[j] = nullptr;
  }
  if (!c.d_ctrl) {
    int r = dalloc(c, &c.d_ctrl, 1);
    if (r) return r;
    CU(cudaMemset(c.d_ctrl, 0, sizeof(CtrlState)));
  }
  if (solve_grid_blocks(c, c.opts.precision == HF_PREC_MIXED ? 1 : 0) < 1)
    return set_err(HF_ECUDA, "no co-resident grid for the persistent solve kernel");
  cudaStream_t cs = nullptr;
  CU(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaStream_t saved = c.stream;
  std::string err;
  auto chk = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && err.empty()) err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaSuccess;
  };
  // one graph per result buffer: the kernels' DevArrays carry it as xout (only these graphs do)
  for (int j = 0; j < 2 && err.empty(); ++j) {
    cudaGraph_t g = nullptr;
    if (chk(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed), "capture")) {
      c.stream = cs;
      c.A.xout = c.d_stage_x[j];
      chk(launch_finalize(c, FIN_RHS, nullptr, 0, 0), "rhs finalize");
      chk(launch_solve(c), "persistent solve");
      chk(launch_stage_fallback(c), "result fallback");
      chk(launch_graph_step_end(c, c.d_ctrl, c.d_sctl), "step end");
      if (c.tempdep) chk(launch_tempdep(c), "properties");
      c.A.xout = nullptr;
      chk(cudaStreamEndCapture(cs, &g), "end capture");
      if (err.empty()) chk(cudaGraphInstantiate(&c.post_exec[j], g, 0), "instantiate");
    }
    c.post_graph[j] = g;
  }
  c.A.xout = nullptr;
  c.stream = saved;
  cudaStreamDestroy(cs);
  if (!err.empty()) {
    for (int j = 0; j < 2; ++j) {
      if (c.post_exec[j]) cudaGraphExecDestroy(c.post_exec[j]);
      if (c.post_graph[j]) cudaGraphDestroy(c.post_graph[j]);
      c.post_exec[j] = nullptr;
      c.post_graph[j] = nullptr;
    }
    cudaGetLastError();
    return set_err(HF_ECUDA, "graph capture: " + err);
  }
  c.post_precision = c.opts.precision;
  c.post_criterion = c.opts.criterion;
  return HF_OK;
}

// Chunks of the host arrays for hf_step_host_async: whole z-slabs of tasks (instance i, task
// planes [bz*zc, (bz+1)*zc)), which are contiguous in the compact host layout, in the device
// layout and in the task table, merged in order into at most kHostChunks chunks of about equal
// cells.
void build_host_chunks(Ctx& c) {
  if (c.host_chunks_depth == c.depth && !c.host_chunks.empty()) return;
  int64_t total = 0;
  for (const auto& d : c.h_inst) total += d.n;
  const int64_t target = (total + Ctx::kHostChunks - 1) / Ctx::kHostChunks;
  c.host_chunks.clear();
  Ctx::HostChunk cur{0, 0, 0, 0, 0, 0};
  bool open = false;
  for (const auto& d : c.h_inst) {
    const int64_t nbx = (d.nx + kTX - 1) / kTX, nby = (d.ny + kTY - 1) / kTY;
    const int64_t nxy = (int64_t)d.nx * d.ny;
    for (int64_t z0 = 0, bz = 0; z0 < d.nz; z0 += d.zc, ++bz) {
      const int64_t z1 = std::min<int64_t>(z0 + d.zc, d.nz);
      const Ctx::HostChunk g{d.hoff + z0 * nxy, d.hoff + z1 * nxy, d.off + z0 * nxy,
                             d.off + z1 * nxy, d.task0 + bz * nbx * nby,
                             d.task0 + (bz + 1) * nbx * nby};
      if (!open) {
        cur = g;
        open = true;
      } else {
        cur.chi = g.chi;
        cur.ghi = g.ghi;
        cur.thi = g.thi;
      }
      if (cur.chi - cur.clo >= target && (int)c.host_chunks.size() < Ctx::kHostChunks - 1) {
        c.host_chunks.push_back(cur);
        open = false;
      }
    }
  }
  if (open) c.host_chunks.push_back(cur);
  c.host_chunks_depth = c.depth;
}

void fill_stats(Ctx& c, hf_stats* st, int64_t steps, const std::vector<InstScal>& before) {
  if (!st) return;
  std::memset(st, 0, sizeof(*st));
  st->steps = steps;
  st->failed_step = -1;
  st->failed_instance = -1;
  for (int64_t i = 0; i < c.ninst; ++i) {
    const InstScal& s = c.h_scal[i];
    const InstScal& b = before[i];
    st->iterations += s.tot_iters - b.tot_iters;
    st->inner_iterations += s.tot_inner - b.tot_inner;
    st->refinements += s.tot_refine - b.tot_refine;
    st->unconverged += s.unconverged - b.unconverged;
    st->last_iter = std::max<int64_t>(st->last_iter, s.last_iter);
    st->last_err = std::max(st->last_err, s.last_err);
    st->last_true_relres = std::max(st->last_true_relres, s.last_relres);
    if (s.status && st->failed_instance < 0) {
      st->failed_instance = (int32_t)i;
      st->failed_step = s.failed_step;
      st->status = status_code(s.status);
    }
  }
}

// The index-check record of the checked build: HF_EDEVICE with the first failed check's site.
int check_record(Ctx& c) {
#ifdef HF_CHECKED
  unsigned long long rec[4] = {0, 0, 0, 0};
  CU(cudaMemcpyAsync(rec, c.A.check, sizeof(rec), cudaMemcpyDeviceToHost, c.stream));
  CU(cudaStreamSynchronize(c.stream));
  if (rec[0])
    return set_err(HF_EDEVICE, "index check failed " + std::to_string(rec[0]) + " time(s); first at "
                               "site " + std::to_string(rec[1]) + " (file " +
                               std::to_string(rec[1] / 100000) + ", line " +
                               std::to_string(rec[1] % 100000) + "): index " +
                               std::to_string((long long)rec[2]) + " outside [0, " +
                               std::to_string(rec[3]) + ")");
#else
  (void)c;
#endif
  return HF_OK;
}

int first_error(Ctx& c) {
  if (int r = check_record(c)) return r;
  for (int64_t i = 0; i < c.ninst; ++i) {
    if (c.h_scal[i].status) return status_code(c.h_scal[i].status);
    if (c.h_scal[i].devcheck)
      return set_err(HF_EDEVICE, "assembly consistency check failed on instance " +
                                     std::to_string(i) + " (code " +
                                     std::to_string(c.h_scal[i].devcheck) + ")");
  }
  return HF_OK;
}

// Copy a per-instance host array (concatenated, unpadded) to a padded device array.
template <typename T>
int upload_padded(Ctx& c, T* dst, const T* src) {
  int64_t pos = 0;
  for (int64_t i = 0; i < c.ninst; ++i) {
    const InstDesc& d = c.h_inst[i];
    CU(cudaMemcpyAsync(dst + d.off, src + pos, sizeof(T) * d.n, cudaMemcpyHostToDevice, c.stream));
    pos += d.n;
  }
  return HF_OK;
}

template <typename T>
int download_padded(Ctx& c, T* dst, const T* src) {
  int64_t pos = 0;
  for (int64_t i = 0; i < c.ninst; ++i) {
    const InstDesc& d = c.h_inst[i];
    CU(cudaMemcpyAsync(dst + pos, src + d.off, sizeof(T) * d.n, cudaMemcpyDeviceToHost, c.stream));
    pos += d.n;
  }
  return HF_OK;
}

// Task depth of the option 0 (default): kZC planes, or fewer (halving down to kMinTaskDepth) while
// the grids would give fewer than two tasks per block of a persistent solve (3 blocks per SM on
// GB300's 152).  A round lasts as long as its slowest task, so on a small grid deep tasks leave
// most SMs idle: a 64^3 grid has 32 tasks of 8192 cells at depth 32, 256 at depth 4; at 128^3
// depth 8 (1024 tasks) solved faster than 16 (512) and 32.  A fixed count keeps the task table,
// and so the bits, independent of the device.
constexpr int64_t kDefaultMinTasks = 2 * 3 * 152;
int effective_depth(const Ctx& c, const hf_solver_opts& o) {
  if (o.task_depth > 0) return o.task_depth;
  for (int depth = kZC; depth > kMinTaskDepth; depth /= 2) {
    int64_t n = 0;
    for (const InstDesc& d : c.h_inst)
      n += (int64_t)((d.nx + kTX - 1) / kTX) * ((d.ny + kTY - 1) / kTY) * ((d.nz + depth - 1) / depth);
    if (n >= kDefaultMinTasks) return depth;
  }
  return kMinTaskDepth;
}

// (Re)build the task table for a task depth: per instance, kTX x kTY column tiles x `depth`
// planes, ordered (z, y, x); uploads the table and the instance descriptors, recomputes the
// per-task heater flags and forgets what depended on the old table (captured graph, grid size).
int build_tasks(Ctx& c, int depth) {
  std::vector<int4> tasks;
  for (int64_t i = 0; i < c.ninst; ++i) {
    InstDesc& d = c.h_inst[i];
    const int nbx = (d.nx + kTX - 1) / kTX, nby = (d.ny + kTY - 1) / kTY;
    const int nbz = (d.nz + depth - 1) / depth;
    d.task0 = (int64_t)tasks.size();
    d.ntask = nbx * nby * nbz;
    d.zc = depth;
    for (int bz = 0; bz < nbz; ++bz)
      for (int by = 0; by < nby; ++by)
        for (int bx = 0; bx < nbx; ++bx)
          tasks.push_back(make_int4((int)i, bx * kTX, by * kTY, bz * depth));
  }
  if ((int64_t)tasks.size() > c.ntasks_cap) return set_err(HF_EARG, "task depth below the minimum");
  c.ntasks = (int64_t)tasks.size();
  c.A.ntasks = c.ntasks;
  std::vector<int32_t> large;
  for (int64_t i = 0; i < c.ninst; ++i)
    if (c.h_inst[i].ntask > kWarpSumMax) large.push_back((int32_t)i);
  c.A.nlarge = (int64_t)large.size();
  c.A.nsmall = c.ninst - c.A.nlarge;
  if (!large.empty())
    CU(cudaMemcpyAsync(const_cast<int32_t*>(c.A.large), large.data(), sizeof(int32_t) * large.size(),
                       cudaMemcpyHostToDevice, c.stream));
  CU(cudaMemcpyAsync(const_cast<int4*>(c.A.tasks), tasks.data(), sizeof(int4) * tasks.size(),
                     cudaMemcpyHostToDevice, c.stream));
  CU(cudaMemcpyAsync(const_cast<InstDesc*>(c.A.inst), c.h_inst.data(), sizeof(InstDesc) * c.ninst,
                     cudaMemcpyHostToDevice, c.stream));
  CU(launch_task_heat(c));
  CU(cudaStreamSynchronize(c.stream));
  c.depth = depth;
  c.solve_blocks[0] = c.solve_blocks[1] = 0;
  drop_graph(c);
  return HF_OK;
}

int create_impl(const hf_problem* probs, int64_t count, const hf_solver_opts* opts, hf_ctx** out) {
  if (!probs || count < 1 || !out) return set_err(HF_EARG, "null problem/out or count < 1");
  *out = nullptr;
  hf_solver_opts o;
  if (opts) o = *opts; else hf_default_opts(&o);
  int rc = validate_opts(o);
  if (rc) return rc;
  for (int64_t i = 0; i < count; ++i) {
    const hf_problem& p = probs[i];
    if (p.nx < 1 || p.ny < 1 || p.nz < 1) return set_err(HF_EARG, "grid dimensions must be >= 1");
    const int64_t n = p.nx * p.ny * p.nz;
    if (n >= (int64_t(1) << 31)) return set_err(HF_EARG, "more than 2^31-1 cells in one grid");
    if ((p.nx + 3) / 4 * 4 * p.ny * p.nz >= (int64_t(1) << 31))
      return set_err(HF_EARG, "more than 2^31-1 cells in one grid with rows padded to 4 cells");
    if (p.nx == 1 && n > 1)
      return set_err(HF_EARG, "nx = 1 with more than one cell: the reference's COO assembly "
                              "(sparse_Hmatrix) writes past its capacity for such grids");
    if (!p.kappa || !p.rho || !p.heat_capacity) return set_err(HF_EARG, "kappa, rho, heat_capacity required");
    if (!(p.time_step > 0.0)) return set_err(HF_EARG, "time_step must be > 0");
    if (!(p.lx > 0.0 && p.ly > 0.0 && p.lz > 0.0)) return set_err(HF_EARG, "box lengths must be > 0");
  }
  hf_ctx* h = new hf_ctx();
  Ctx& c = h->c;
  c.opts = o;
  if (cudaGetDevice(&c.device) != cudaSuccess) { delete h; return set_err(HF_ECUDA, "no CUDA device"); }
  if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return set_err(HF_ECUDA, "cudaStreamCreate failed");
  }
  c.own_stream = true;
  c.ninst = count;
  // ---- layout: instances at multiples of kTile cells
  int64_t off = 0, tiles = 0, hoff = 0, off4 = 0;
  std::vector<int32_t> tile_inst;
  c.h_inst.resize(count);
  c.h_bc.resize(count);
  for (int64_t i = 0; i < count; ++i) {
    const hf_problem& p = probs[i];
    InstDesc& d = c.h_inst[i];
    std::memset(&d, 0, sizeof(d));
    d.nx = (int32_t)p.nx; d.ny = (int32_t)p.ny; d.nz = (int32_t)p.nz;
    d.n = (int32_t)(p.nx * p.ny * p.nz);
    d.off = off;
    d.hoff = hoff;
    hoff += d.n;
    d.sx = (int32_t)((p.nx + 3) / 4 * 4);
    d.off4 = off4;
    const int64_t n4 = (int64_t)d.sx * p.ny * p.nz;
    off4 += (n4 + kTile - 1) / kTile * kTile;
    d.tile0 = tiles;
    d.ntiles = (int32_t)((d.n + kTile - 1) / kTile);
    for (int t = 0; t < d.ntiles; ++t) tile_inst.push_back((int32_t)i);
    tiles += d.ntiles;
    off += (int64_t)d.ntiles * kTile;
    d.px = p.periodic[0] ? 1 : 0; d.py = p.periodic[1] ? 1 : 0; d.pz = p.periodic[2] ? 1 : 0;
    d.icattaneo = p.icattaneo; d.isteady = p.isteady;
    d.qdens_mode = p.qdens_mode;
    d.time_step = p.time_step;
    d.inv_dt = 1.0 / p.time_step;                       // mod_setup.f90:45
    d.freq = p.freq;
    d.power_in = p.power_in;
    d.time_pulse = (double)p.heated_steps * p.time_step; // mod_heating.f90:41
    d.t_bath = p.t_bath;
    // Length = L/real(n) (default-real conversion of n), volume = L1*L2*L3 (mod_inputs.f90:619-622)
    d.len[0] = p.lx / (double)(float)p.nx;
    d.len[1] = p.ly / (double)(float)p.ny;
    d.len[2] = p.lz / (double)(float)p.nz;
    d.volume = d.len[0] * d.len[1] * d.len[2];
    double hv = 0.0;
    bool heater = false, case5 = false, em = false;
    for (int64_t k = 0; k < d.n; ++k) {
      int64_t ih = p.iheater ? p.iheater[k] : 0;
      if (ih > 0) { heater = true; hv = hv + d.volume; }   // mod_heating.f90:145-148
      if (ih == 5) case5 = true;
      if (p.em && p.em[k] != 0.0) em = true;
    }
    d.heater = heater ? 1 : 0;
    d.has_case5 = case5 ? 1 : 0;
    d.has_em = (heater && em) ? 1 : 0;
    d.has_power = (heater && p.power) ? 1 : 0;
    d.heated_volume = hv;
    InstBC& bc = c.h_bc[i];
    for (int f = 0; f < 6; ++f) {
      bc.kb[f] = p.kappa_bound[f];
      bc.tb[f] = p.t_bath_face[f];
      bc.cg[f] = p.cg_face[f] ? 1 : 0;
      bc.pd[f] = 0.0;
    }
    bc.br = p.br;
    // Neumann power densities, mod_boundary.f90:43-66 (T_BathCG / (volume * n_a * n_b))
    const double nxd = (double)p.nx, nyd = (double)p.ny, nzd = (double)p.nz;
    if (bc.cg[4]) bc.pd[4] = p.t_bath_cg / (d.volume * nxd * nyd);
    if (bc.cg[5]) bc.pd[5] = p.t_bath_cg / (d.volume * nxd * nyd);
    if (bc.cg[2]) bc.pd[2] = p.t_bath_cg / (d.volume * nxd * nzd);
    if (bc.cg[3]) bc.pd[3] = p.t_bath_cg / (d.volume * nxd * nzd);
    if (bc.cg[0]) bc.pd[0] = p.t_bath_cg / (d.volume * nyd * nzd);
    if (bc.cg[1]) bc.pd[1] = p.t_bath_cg / (d.volume * nyd * nzd);
    c.any_heater |= heater;
    c.any_power |= (heater && p.power);
    c.any_em |= (heater && em);
    c.any_case5 |= case5;
  }
  c.ncells = off;
  c.ntiles = tiles;
  // task buffers are sized for the shallowest task depth; the table itself is built later
  c.ntasks_cap = 0;
  for (int64_t i = 0; i < count; ++i) {
    const InstDesc& d = c.h_inst[i];
    c.ntasks_cap += (int64_t)((d.nx + kTX - 1) / kTX) * ((d.ny + kTY - 1) / kTY) *
                    ((d.nz + kMinTaskDepth - 1) / kMinTaskDepth);
  }
  c.ntasks = c.ntasks_cap;
  const size_t N = (size_t)c.ncells;
  const size_t N4 = (size_t)off4;   // cells of the FP32 inner-solve layout
  // ---- device memory
  DevArrays& A = c.A;
  std::memset(&A, 0, sizeof(A));
  A.ncells = c.ncells; A.ntiles = c.ntiles; A.ninst = c.ninst;
  A.opts = dev_opts(o);
#define ALLOC(ptr, n) do { int r_ = dalloc(c, &(ptr), (n)); if (r_) { free_all(c); delete h; return r_; } } while (0)
  InstDesc* d_inst; InstScal* d_scal; int32_t* d_tile_inst;
  ALLOC(d_inst, (size_t)count);
  ALLOC(d_scal, (size_t)count);
  ALLOC(d_tile_inst, (size_t)tiles);
  int8_t* d_task_heat;
  int4* d_tasks;
  ALLOC(d_task_heat, (size_t)c.ntasks);
  ALLOC(d_tasks, (size_t)c.ntasks);
  A.task_heat = d_task_heat;
  A.tasks = d_tasks;
  A.ntasks = c.ntasks;
  ALLOC(A.partials, (size_t)c.ntasks * kNR);
  ALLOC(c.d_sctl, (size_t)1);
  ALLOC(A.counters, (size_t)count);
  ALLOC(c.d_bc, (size_t)count);
  int32_t* d_large;
  ALLOC(d_large, (size_t)count);
  A.large = d_large;
  A.inst = d_inst; A.scal = d_scal; A.tile_inst = d_tile_inst;
  ALLOC(A.diag, N); ALLOC(A.cx, N); ALLOC(A.cy, N); ALLOC(A.cz, N); ALLOC(A.sinv, N);
  ALLOC(A.rsum, N); ALLOC(A.sinv32, N);
  ALLOC(A.a64x, N); ALLOC(A.a64y, N); ALLOC(A.a64z, N);
  ALLOC(A.a32x, N4); ALLOC(A.a32y, N4); ALLOC(A.a32z, N4);
  ALLOC(A.rhoc, N); ALLOC(A.ccat, N); ALLOC(A.bvec, N); ALLOC(A.tau_s, N); ALLOC(A.scoef, N);
  ALLOC(c.asm_.kappa, N);
  if (c.any_power) ALLOC(A.power, N);
  if (c.any_em) ALLOC(A.emc, N);
  if (c.any_heater) ALLOC(A.icase, N);
  for (int k = 0; k < 4; ++k) ALLOC(A.tbuf[k], N);
  ALLOC(A.hx[0], N); ALLOC(A.hx[1], N);
  ALLOC(A.stamps, (size_t)kStamps);
  ALLOC(A.check, (size_t)4);
  ALLOC(A.b, N); ALLOC(A.y, N); ALLOC(A.r, N); ALLOC(A.p, N); ALLOC(A.q, N); ALLOC(A.p2, N);
  ALLOC(A.y32, N4); ALLOC(A.r32, N4); ALLOC(A.p32, N4); ALLOC(A.q32, N4); ALLOC(A.p232, N4);
  double *d_rho, *d_hc, *d_tau, *d_em = nullptr;
  ALLOC(d_rho, N); ALLOC(d_hc, N); ALLOC(d_tau, N);
  if (c.any_em) ALLOC(d_em, N);
#undef ALLOC
  if (cudaMallocHost((void**)&c.h_scal, sizeof(InstScal) * count) != cudaSuccess) {
    free_all(c); delete h; return set_err(HF_ENOMEM, "cudaMallocHost failed");
  }
  auto fail = [&](int r) { free_all(c); delete h; return r; };
#define CK(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) return fail(set_err(HF_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_))); } while (0)
  CK(cudaMemsetAsync(A.counters, 0, sizeof(unsigned) * count, c.stream));
  CK(cudaMemsetAsync(d_scal, 0, sizeof(InstScal) * count, c.stream));
  CK(cudaMemsetAsync(c.d_sctl, 0, sizeof(SolveCtl), c.stream));
  CK(cudaMemsetAsync(A.stamps, 0, sizeof(unsigned long long) * kStamps, c.stream));
  CK(cudaMemsetAsync(A.check, 0, sizeof(unsigned long long) * 4, c.stream));
  for (void* p : {(void*)A.diag, (void*)A.cx, (void*)A.cy, (void*)A.cz, (void*)c.asm_.kappa,
                  (void*)d_rho, (void*)d_hc, (void*)d_tau, (void*)A.rhoc, (void*)A.ccat, (void*)A.scoef,
                  (void*)A.bvec, (void*)A.tau_s, (void*)A.a64x, (void*)A.a64y, (void*)A.a64z,
                  (void*)A.b, (void*)A.y, (void*)A.r, (void*)A.p, (void*)A.q, (void*)A.rsum,
                  (void*)A.p2, (void*)A.hx[0], (void*)A.hx[1]})
    CK(cudaMemsetAsync(p, 0, N * sizeof(double), c.stream));
  // the padding cells of the FP32 layout stay zero: no kernel writes them anything else
  for (void* p : {(void*)A.a32x, (void*)A.a32y, (void*)A.a32z, (void*)A.y32, (void*)A.r32,
                  (void*)A.p32, (void*)A.q32, (void*)A.p232})
    CK(cudaMemsetAsync(p, 0, N4 * sizeof(float), c.stream));
  CK(cudaMemsetAsync(A.sinv32, 0, N * sizeof(float), c.stream));
  for (int k = 0; k < 4; ++k) CK(cudaMemsetAsync(A.tbuf[k], 0, N * sizeof(double), c.stream));
  if (d_em) CK(cudaMemsetAsync(d_em, 0, N * sizeof(double), c.stream));
  if (A.power) CK(cudaMemsetAsync(A.power, 0, N * sizeof(double), c.stream));
  if (A.icase) CK(cudaMemsetAsync(A.icase, 0, N, c.stream));
  CK(cudaMemcpyAsync(d_inst, c.h_inst.data(), sizeof(InstDesc) * count, cudaMemcpyHostToDevice, c.stream));
  CK(cudaMemcpyAsync(c.d_bc, c.h_bc.data(), sizeof(InstBC) * count, cudaMemcpyHostToDevice, c.stream));
  CK(cudaMemcpyAsync(d_tile_inst, tile_inst.data(), sizeof(int32_t) * tiles, cudaMemcpyHostToDevice, c.stream));
  // per-cell inputs into the padded layout
  std::vector<int8_t> icase;
  for (int64_t i = 0; i < count; ++i) {
    const hf_problem& p = probs[i];
    const InstDesc& d = c.h_inst[i];
    CK(cudaMemcpyAsync(c.asm_.kappa + d.off, p.kappa, 8 * d.n, cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(d_rho + d.off, p.rho, 8 * d.n, cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(d_hc + d.off, p.heat_capacity, 8 * d.n, cudaMemcpyHostToDevice, c.stream));
    if (p.tau) CK(cudaMemcpyAsync(d_tau + d.off, p.tau, 8 * d.n, cudaMemcpyHostToDevice, c.stream));
    if (d_em && p.em) CK(cudaMemcpyAsync(d_em + d.off, p.em, 8 * d.n, cudaMemcpyHostToDevice, c.stream));
    if (A.power) {
      if (p.power) {
        CK(cudaMemcpyAsync(A.power + d.off, p.power, 8 * d.n, cudaMemcpyHostToDevice, c.stream));
      } else {
        std::vector<double> pw((size_t)d.n, p.power_in);
        CK(cudaMemcpyAsync(A.power + d.off, pw.data(), 8 * d.n, cudaMemcpyHostToDevice, c.stream));
        CK(cudaStreamSynchronize(c.stream));
      }
    }
    if (A.icase) {
      icase.assign((size_t)d.n, 0);
      for (int64_t k = 0; k < d.n; ++k) {
        int64_t ih = p.iheater ? p.iheater[k] : 0;
        icase[k] = (int8_t)(ih < 0 ? -1 : (ih > 6 ? 7 : ih));
      }
      CK(cudaMemcpyAsync(A.icase + d.off, icase.data(), d.n, cudaMemcpyHostToDevice, c.stream));
      CK(cudaStreamSynchronize(c.stream));
    }
  }
  {
    const int r = build_tasks(c, effective_depth(c, o));
    if (r) return fail(r);
  }
  CK(launch_props(c, d_rho, d_hc, d_tau, d_em));
  CK(launch_assemble(c));
  CK(cudaStreamSynchronize(c.stream));
  // mean of sinv over a strided sample of each instance (scaling of FP32 right-hand sides)
  for (int64_t i = 0; i < count; ++i) {
    InstDesc& d = c.h_inst[i];
    const int64_t m = std::min<int64_t>(d.n, 4096);
    const int64_t stride = d.n / m;
    std::vector<double> smp((size_t)m);
    CK(cudaMemcpy2D(smp.data(), sizeof(double), A.sinv + d.off, sizeof(double) * stride,
                    sizeof(double), (size_t)m, cudaMemcpyDeviceToHost));
    double acc = 0.0;
    for (double v : smp) acc += v;
    d.mean_sinv = acc / (double)m;
  }
  CK(cudaMemcpyAsync(d_inst, c.h_inst.data(), sizeof(InstDesc) * count, cudaMemcpyHostToDevice, c.stream));
  // initial scalars: roles 0..3, status from assembly
  CK(cudaMemcpyAsync(c.h_scal, d_scal, sizeof(InstScal) * count, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  for (int64_t i = 0; i < count; ++i) {
    InstScal& s = c.h_scal[i];
    s.role[0] = 0; s.role[1] = 1; s.role[2] = 2; s.role[3] = 3;
    s.sigma = 1.0; s.sigma_prev = 1.0;
    s.failed_step = -1;
  }
  CK(cudaMemcpyAsync(d_scal, c.h_scal, sizeof(InstScal) * count, cudaMemcpyHostToDevice, c.stream));
  CK(cudaStreamSynchronize(c.stream));
#undef CK
  // the temporary property inputs are no longer needed
  for (void* p : {(void*)d_rho, (void*)d_hc, (void*)d_tau, (void*)d_em}) {
    if (!p) continue;
    cudaFree(p);
    c.allocs.erase(std::remove(c.allocs.begin(), c.allocs.end(), p), c.allocs.end());
  }
  for (int64_t i = 0; i < count; ++i) {
    if (c.h_scal[i].devcheck) {
      int r = set_err(HF_EDEVICE, "assembly consistency check failed (code " +
                                      std::to_string(c.h_scal[i].devcheck) + ", instance " +
                                      std::to_string(i) + "): operator diagonal must be < 0");
      free_all(c);
      delete h;
      return r;
    }
  }
  *out = h;
  return HF_OK;
}

}  // namespace

extern "C" {

int hf_create(const hf_problem* prob, const hf_solver_opts* opts, hf_ctx** out) {
  return create_impl(prob, 1, opts, out);
}

int hf_create_batch(const hf_problem* probs, int64_t count, const hf_solver_opts* opts, hf_ctx** out) {
  return create_impl(probs, count, opts, out);
}

int hf_destroy(hf_ctx* h) {
  if (!h) return HF_OK;
  cudaStreamSynchronize(h->c.stream);
  free_all(h->c);
  delete h;
  return HF_OK;
}

int hf_set_opts(hf_ctx* h, const hf_solver_opts* opts) {
  if (!h || !opts) return set_err(HF_EARG, "null argument");
  if (h->c.async_pending)
    return set_err(HF_ESTATE, "host-buffer steps are queued: call hf_host_sync first");
  int rc = validate_opts(*opts);
  if (rc) return rc;
  h->c.opts = *opts;
  h->c.A.opts = dev_opts(*opts);
  drop_graph(h->c);   // captured kernels hold the options by value
  if (effective_depth(h->c, *opts) != h->c.depth) return build_tasks(h->c, effective_depth(h->c, *opts));
  return HF_OK;
}

int hf_get_sizes(const hf_ctx* h, int64_t* instances, int64_t* total_cells) {
  if (!h) return set_err(HF_EARG, "null context");
  int64_t tot = 0;
  for (const auto& d : h->c.h_inst) tot += d.n;
  if (instances) *instances = h->c.ninst;
  if (total_cells) *total_cells = tot;
  return HF_OK;
}

int64_t hf_instance_cells(const hf_ctx* h, int64_t i) {
  if (!h || i < 0 || i >= h->c.ninst) return -1;
  return h->c.h_inst[i].n;
}

int hf_set_stream(hf_ctx* h, void* stream) {
  if (!h) return set_err(HF_EARG, "null context");
  Ctx& c = h->c;
  if (int r_ = refuse_queued(c)) return r_;
  CU(cudaStreamSynchronize(c.stream));
  if (stream) {
    if (c.own_stream) cudaStreamDestroy(c.stream);
    c.stream = (cudaStream_t)stream;
    c.own_stream = false;
  } else if (!c.own_stream) {
    CU(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    c.own_stream = true;
  }
  return HF_OK;
}

int hf_set_state(hf_ctx* h, const double* tp, const double* tpp) {
  if (!h || !tp || !tpp) return set_err(HF_EARG, "null argument");
  Ctx& c = h->c;
  int rc = sync_scal(c);
  if (rc) return rc;
  int64_t pos = 0;
  for (int64_t i = 0; i < c.ninst; ++i) {
    const InstDesc& d = c.h_inst[i];
    const InstScal& s = c.h_scal[i];
    CU(cudaMemcpyAsync(c.A.tbuf[s.role[0]] + d.off, tp + pos, 8 * d.n, cudaMemcpyHostToDevice, c.stream));
    CU(cudaMemcpyAsync(c.A.tbuf[s.role[1]] + d.off, tpp + pos, 8 * d.n, cudaMemcpyHostToDevice, c.stream));
    pos += d.n;
  }
  c.state_set = true;
  return push_scal(c);   // a new state: the stored products H T are stale
}

int hf_get_state(hf_ctx* h, double* tp, double* tpp) {
  if (!h) return set_err(HF_EARG, "null context");
  Ctx& c = h->c;
  int rc = sync_scal(c);
  if (rc) return rc;
  int64_t pos = 0;
  for (int64_t i = 0; i < c.ninst; ++i) {
    const InstDesc& d = c.h_inst[i];
    const InstScal& s = c.h_scal[i];
    if (tp) CU(cudaMemcpyAsync(tp + pos, c.A.tbuf[s.role[0]] + d.off, 8 * d.n, cudaMemcpyDeviceToHost, c.stream));
    if (tpp) CU(cudaMemcpyAsync(tpp + pos, c.A.tbuf[s.role[1]] + d.off, 8 * d.n, cudaMemcpyDeviceToHost, c.stream));
    pos += d.n;
  }
  CU(cudaStreamSynchronize(c.stream));
  return HF_OK;
}

int hf_state_device(hf_ctx* h, double** tp, double** tpp) {
  if (!h) return set_err(HF_EARG, "null context");
  Ctx& c = h->c;
  if (c.ninst != 1) return set_err(HF_EARG, "device state pointers are for single-grid contexts");
  int rc = sync_scal(c);
  if (rc) return rc;
  if (tp) *tp = c.A.tbuf[c.h_scal[0].role[0]];
  if (tpp) *tpp = c.A.tbuf[c.h_scal[0].role[1]];
  return HF_OK;
}

int hf_state_device_ready(hf_ctx* h) {
  if (!h) return set_err(HF_EARG, "null context");
  h->c.state_set = true;
  int rc = sync_scal(h->c);
  if (rc) return rc;
  return push_scal(h->c);   // the state was written in place: the stored products H T are stale
}

int hf_step(hf_ctx* h, int64_t itime, hf_stats* stats) {
  return hf_run(h, itime, 1, stats);
}

}  // extern "C"
namespace {
int run_steps(Ctx& c, int64_t itime0, int64_t nsteps, hf_stats* stats);
}
extern "C" {

int hf_run(hf_ctx* h, int64_t itime0, int64_t nsteps, hf_stats* stats) {
  if (!h || nsteps < 0) return set_err(HF_EARG, "null context or nsteps < 0");
  return run_steps(h->c, itime0, nsteps, stats);
}

}  // extern "C"

namespace {
// Device-side view of a pinned (page-locked, mapped) host array, or null.
double* pinned_view(const void* p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
  if (((uintptr_t)at.devicePointer & 7u) != 0u) return nullptr;
  return static_cast<double*>(at.devicePointer);
}
}  // namespace

extern "C" {

int hf_step_host_async(hf_ctx* h, int64_t itime, const double* tp, const double* tpp, double* out) {
  if (!h || !tp || !tpp || !out) return set_err(HF_EARG, "null argument");
  Ctx& c = h->c;
  if (!pinned_view(tp) || !pinned_view(tpp) || !pinned_view(out))
    return set_err(HF_EARG, "hf_step_host_async: tp, tpp and out must be pinned host memory "
                            "(cudaHostAlloc, or hf_host_register)");
  if (c.opts.use_graph != 1 && c.opts.use_graph != 3)
    return set_err(HF_EARG, "hf_step_host_async: needs use_graph 1 or 3 (captured steps)");
  int64_t total = 0;
  for (const auto& d : c.h_inst) total += d.n;
  int rc;
  if (!c.async_pending) {            // first step of a queue: nothing of ours is in flight
    if ((rc = sync_scal(c))) return rc;
    c.async_before.assign(c.h_scal, c.h_scal + c.ninst);
    c.async_steps = 0;
    c.async_calls.clear();
    c.async_host_kernels = 0;
    for (int j = 0; j < 2; ++j) {   // the result buffers are part of the post-RHS graphs
      if (!c.d_stage_x[j] && (rc = dalloc(c, &c.d_stage_x[j], (size_t)total))) return rc;
      if (!c.stage_x_free[j]) CU(cudaEventCreateWithFlags(&c.stage_x_free[j], cudaEventDisableTiming));
      CU(cudaEventRecord(c.stage_x_free[j], c.stream));
    }
    if ((rc = build_post_graph(c))) return rc;
    build_host_chunks(c);
    if (!c.copy_stream) CU(cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking));
    if (!c.out_stream) CU(cudaStreamCreateWithFlags(&c.out_stream, cudaStreamNonBlocking));
    if (!c.ev_gathered) CU(cudaEventCreateWithFlags(&c.ev_gathered, cudaEventDisableTiming));
    for (auto& o : c.outs) {
      if (!o.done) CU(cudaEventCreateWithFlags(&o.done, cudaEventDisableTiming));
      for (auto& e : o.chunk)
        if (!e) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    for (auto& st : c.stage) {
      for (cudaEvent_t* e : {&st.in_pp, &st.free})
        if (!*e) CU(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
      for (auto& e : st.in_chunk)
        if (!e) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      for (double** b : {&st.p, &st.pp})
        if (!*b && (rc = dalloc(c, b, (size_t)total))) return rc;
      CU(cudaEventRecord(st.free, c.stream));
    }
    if (!c.d_check_call && (rc = dalloc(c, &c.d_check_call, (size_t)1))) return rc;
    const int64_t none = INT64_MAX;
    CU(cudaMemcpyAsync(c.d_check_call, &none, sizeof(none), cudaMemcpyHostToDevice, c.stream));
    for (auto& o : c.outs) {
      CU(cudaEventRecord(o.done, c.stream));
      o.ptr = nullptr;
    }
  }
  const std::vector<Ctx::HostChunk>& ch = c.host_chunks;
  const int nch = (int)ch.size();
  const int64_t call = c.async_steps;
  Ctx::Stage& st = c.stage[call & 1];
  // Early start: the inputs are the previous call's result and the previous call's T^n -- the
  // rotation simulate() performs -- so, unless the caller broke the rule that queued arrays stay
  // untouched, their bits are those the device holds as T^n and T^(n-1) now.  The step then starts
  // from the device's copy while the uploads travel, and the next call (or hf_host_sync) compares
  // the uploaded bits with that copy before the copy can be overwritten; a difference makes
  // hf_host_sync run the queue again from that call's uploaded inputs.
  const bool early = call >= 1 && tp == c.outs[c.out_last].ptr && tpp == c.async_calls.back().tp;
  // Copy stream.  A staging set is free once the consumer of its previous inputs (two calls back)
  // has run; by then every download older than the last kHostOuts queued ones is done (the main
  // stream had waited, before that call's post-RHS graph, for the download of two calls before
  // it, whose result buffer the graph rewrites).  An input that is the destination of one of
  // those downloads waits for it: T^(n-1), normally the result of two steps back, as a whole (its
  // upload then overlaps the previous step's solve); T^n, normally the previous step's result,
  // chunk by chunk behind that chunk's download, so both directions of the link run at once.
  CU(cudaStreamWaitEvent(c.copy_stream, st.free, 0));
  for (const auto& o : c.outs)
    if (o.ptr && tpp == o.ptr) CU(cudaStreamWaitEvent(c.copy_stream, o.done, 0));
  CU(cudaMemcpyAsync(st.pp, tpp, sizeof(double) * (size_t)total, cudaMemcpyHostToDevice,
                     c.copy_stream));
  CU(cudaEventRecord(st.in_pp, c.copy_stream));
  for (int k = 0; k < nch; ++k) {
    for (const auto& o : c.outs)
      if (o.ptr && tp == o.ptr) CU(cudaStreamWaitEvent(c.copy_stream, o.chunk[k], 0));
    CU(cudaMemcpyAsync(st.p + ch[k].clo, tp + ch[k].clo,
                       sizeof(double) * (size_t)(ch[k].chi - ch[k].clo), cudaMemcpyHostToDevice,
                       c.copy_stream));
    CU(cudaEventRecord(st.in_chunk[k], c.copy_stream));
  }
  // Main stream.  First the check of the previous call's inputs if it started early: its step
  // has ended, so its T^n and T^(n-1) are roles 1 and 2 now, and this step's RHS is about to
  // overwrite role 2.
  if (call >= 1 && c.async_calls.back().early) {
    Ctx::Stage& ps = c.stage[(call - 1) & 1];
    CU(cudaStreamWaitEvent(c.stream, ps.in_pp, 0));
    for (int k = 0; k < nch; ++k) CU(cudaStreamWaitEvent(c.stream, ps.in_chunk[k], 0));
    CU(launch_host_check(c, ps.p, ps.pp, call - 1, c.d_check_call, c.stream));
    CU(cudaEventRecord(ps.free, c.stream));
    c.async_host_kernels += 1;
  }
  const int64_t per = c.opts.precision == HF_PREC_MIXED ? c.opts.inner_itmax : c.opts.itmax;
  if (early) {
    // begin the step from the device's copy of the inputs; the whole RHS as one launch
    CU(launch_ctrl_init(c, itime, 2 * (int64_t)(c.opts.max_refine + 3) * (per + 3)));
    CU(launch_graph_step_begin(c, c.d_ctrl, 1 + 5 + (c.tempdep ? 4 : 0)));
    CU(launch_rhs(c));
    c.async_host_kernels += 1;                    // control reset
  } else {
    // place T^(n-1), begin the step, then place each chunk of T^n as it lands and run the RHS of
    // its tasks (the later chunks are still on the link)
    CU(cudaStreamWaitEvent(c.stream, st.in_pp, 0));
    CU(launch_host_in(c, st.pp, 1, c.stream));
    CU(launch_ctrl_init(c, itime, 2 * (int64_t)(c.opts.max_refine + 3) * (per + 3)));
    // kernels of the step outside the host copies: begin, RHS per chunk, finalize, solve, result
    // fallback, end
    CU(launch_graph_step_begin(c, c.d_ctrl, nch + 5 + (c.tempdep ? 4 : 0)));
    for (int k = 0; k < nch; ++k) {
      CU(cudaStreamWaitEvent(c.stream, st.in_chunk[k], 0));
      CU(launch_host_in_range(c, st.p, 0, ch[k].glo, ch[k].ghi, c.stream));
      CU(launch_rhs_range(c, ch[k].tlo, ch[k].thi));
    }
    CU(cudaEventRecord(st.free, c.stream));
    c.async_host_kernels += 2 + nch;              // placements, control reset
  }
  // the rest of the step as one graph, whose last residual sweep also stores the result into
  // d_stage_x[call & 1] (free once the download of two calls back has read it); the download
  // runs on a stream of its own, chunk by chunk, so the next step's work does not queue behind it
  const int xj = (int)(call & 1);
  CU(cudaStreamWaitEvent(c.stream, c.stage_x_free[xj], 0));
  CU(cudaGraphLaunch(c.post_exec[xj], c.stream));
  CU(cudaEventRecord(c.ev_gathered, c.stream));
  CU(cudaStreamWaitEvent(c.out_stream, c.ev_gathered, 0));
  const int next = (c.out_last + 1) % Ctx::kHostOuts;   // replaces the oldest tracked download
  Ctx::HostOut& o = c.outs[next];
  for (int k = 0; k < nch; ++k) {
    CU(cudaMemcpyAsync(out + ch[k].clo, c.d_stage_x[xj] + ch[k].clo,
                       sizeof(double) * (size_t)(ch[k].chi - ch[k].clo), cudaMemcpyDeviceToHost,
                       c.out_stream));
    CU(cudaEventRecord(o.chunk[k], c.out_stream));
  }
  CU(cudaEventRecord(o.done, c.out_stream));
  CU(cudaEventRecord(c.stage_x_free[xj], c.out_stream));
  o.ptr = out;
  c.out_last = next;
  c.async_calls.push_back(Ctx::HostCall{itime, tp, tpp, out, early});
  c.async_pending = true;
  c.async_steps += 1;
  c.state_set = true;
  return HF_OK;
}

int hf_host_sync(hf_ctx* h, hf_stats* stats) {
  if (!h) return set_err(HF_EARG, "null context");
  Ctx& c = h->c;
  if (!c.async_pending) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    return HF_OK;
  }
  const int nch = (int)c.host_chunks.size();
  if (c.async_calls.back().early) {          // the check of the last call's inputs
    Ctx::Stage& ps = c.stage[(c.async_steps - 1) & 1];
    CU(cudaStreamWaitEvent(c.stream, ps.in_pp, 0));
    for (int k = 0; k < nch; ++k) CU(cudaStreamWaitEvent(c.stream, ps.in_chunk[k], 0));
    CU(launch_host_check(c, ps.p, ps.pp, c.async_steps - 1, c.d_check_call, c.stream));
    CU(cudaEventRecord(ps.free, c.stream));
    c.async_host_kernels += 1;
  }
  c.async_pending = false;
  CtrlState cs{};
  int64_t first_bad = INT64_MAX;
  CU(cudaMemcpyAsync(&cs, c.d_ctrl, sizeof(cs), cudaMemcpyDeviceToHost, c.stream));
  CU(cudaMemcpyAsync(&first_bad, c.d_check_call, sizeof(first_bad), cudaMemcpyDeviceToHost, c.stream));
  CU(cudaStreamSynchronize(c.stream));
  CU(cudaStreamSynchronize(c.copy_stream));
  CU(cudaStreamSynchronize(c.out_stream));
  const int64_t steps = c.async_steps;
  c.async_steps = 0;
  c.launches += cs.launches + c.async_host_kernels;
  if (cs.guard_hit & 2)
    return set_err(HF_EDEVICE, "persistent solve: a grid barrier wait reached its time limit");
  if (cs.guard_hit) return set_err(HF_EDEVICE, "captured solve loop reached its iteration bound");
  int rc;
  if (first_bad != INT64_MAX) {
    // An early-started call's uploaded inputs differed from the device copy it started from (a
    // queued array was changed): from that call on, every step runs again from its own uploaded
    // inputs (hf_set_state, one step, the result into its array), as a call without an early
    // start would have.  The queued arrays are still valid: they stay untouched until now.
    for (size_t j = (size_t)first_bad; j < c.async_calls.size(); ++j) {
      const Ctx::HostCall& hc = c.async_calls[j];
      if ((rc = hf_set_state(h, hc.tp, hc.tpp))) return rc;
      hf_stats one;
      if ((rc = run_steps(c, hc.itime, 1, &one))) return rc;
      if ((rc = hf_get_state(h, hc.out, nullptr))) return rc;
    }
    const int64_t none = INT64_MAX;
    CU(cudaMemcpy(c.d_check_call, &none, sizeof(none), cudaMemcpyHostToDevice));
  }
  if ((rc = sync_scal(c))) return rc;
  if ((rc = diagnose(c))) return rc;
  fill_stats(c, stats, steps, c.async_before);
  if (stats) stats->kernel_launches = cs.launches + c.async_host_kernels;
  return first_error(c);
}

int hf_host_register(void* ptr, size_t bytes) {
  if (!ptr || bytes == 0) return set_err(HF_EARG, "null pointer or zero size");
  cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterMapped | cudaHostRegisterPortable);
  if (e != cudaSuccess) return set_err(HF_ECUDA, std::string("cudaHostRegister: ") + cudaGetErrorString(e));
  return HF_OK;
}

int hf_host_unregister(void* ptr) {
  if (!ptr) return set_err(HF_EARG, "null pointer");
  cudaError_t e = cudaHostUnregister(ptr);
  if (e != cudaSuccess) return set_err(HF_ECUDA, std::string("cudaHostUnregister: ") + cudaGetErrorString(e));
  return HF_OK;
}

}  // extern "C"

namespace {
int run_steps(Ctx& c, int64_t itime0, int64_t nsteps, hf_stats* stats) {
  if (!c.state_set) return set_err(HF_ESTATE, "hf_set_state must be called before stepping");
  int rc = sync_scal(c);
  if (rc) return rc;
  std::vector<InstScal> before(c.h_scal, c.h_scal + c.ninst);
  const int64_t launches0 = c.launches;
  int64_t done = 0;
  if (c.opts.use_graph && nsteps > 0) {
    if ((rc = build_graph(c))) return rc;
    const bool loop = c.opts.use_graph == 1 && build_loop_graph(c) == HF_OK;   // 3: per-step graphs
    const bool fp32 = c.opts.precision == HF_PREC_MIXED;
    const int64_t per = fp32 ? c.opts.inner_itmax : c.opts.itmax;
    CtrlState cs{};
    cs.itime = itime0;
    cs.itime_end = itime0 + nsteps;
    cs.limit = 2 * (int64_t)(c.opts.max_refine + 3) * (per + 3);
    CU(cudaMemcpyAsync(c.d_ctrl, &cs, sizeof(cs), cudaMemcpyHostToDevice, c.stream));
    if (loop) {
      CU(cudaGraphLaunch(c.loop_exec, c.stream));                    // the whole time loop
    } else {
      for (int64_t k = 0; k < nsteps; ++k) CU(cudaGraphLaunch(c.graph_exec, c.stream));
    }
    CU(cudaMemcpyAsync(&cs, c.d_ctrl, sizeof(cs), cudaMemcpyDeviceToHost, c.stream));
    CU(cudaStreamSynchronize(c.stream));
    if (cs.guard_hit & 2)
      return set_err(HF_EDEVICE, "persistent solve: a grid barrier wait reached its time limit");
    if (cs.guard_hit) return set_err(HF_EDEVICE, "captured solve loop reached its iteration bound");
    c.launches += cs.launches;
    done = nsteps;
    nsteps = 0;
  }
  for (int64_t k = 0; k < nsteps; ++k) {
    rc = run_one_step(c, itime0 + k);
    if (rc) return rc;
    ++done;
    if (c.ninst == 1) {
      if (c.h_scal[0].status) break;   // the reference stops at the first fatal error
    }
  }
  rc = sync_scal(c);
  if (rc) return rc;
  if ((rc = diagnose(c))) return rc;
  fill_stats(c, stats, done, before);
  if (stats) stats->kernel_launches = c.launches - launches0;
  return first_error(c);
}

// Saved temperature state, stored products H T and scalars of all instances (autotuner).
struct Snapshot {
  double* t = nullptr;   // [T^n | T^(n-1) | H T^n | H T^(n-1)] of every instance, cells in order
  std::vector<InstScal> scal;
};
// Field k of instance i in the context: T^n, T^(n-1), H T^n, H T^(n-1).
double* snapshot_field(Ctx& c, const InstScal& s, int k) {
  if (k < 2) return c.A.tbuf[s.role[k]];
  return c.A.hx[k == 2 ? s.hx_role : 1 - s.hx_role];
}
int snapshot_take(Ctx& c, Snapshot& sn) {
  int rc = sync_scal(c);
  if (rc) return rc;
  sn.scal.assign(c.h_scal, c.h_scal + c.ninst);
  CU(cudaMalloc((void**)&sn.t, sizeof(double) * 4 * (size_t)c.ncells));
  for (int64_t i = 0; i < c.ninst; ++i) {
    const InstDesc& d = c.h_inst[i];
    for (int k = 0; k < 4; ++k)
      CU(cudaMemcpyAsync(sn.t + k * c.ncells + d.off, snapshot_field(c, sn.scal[i], k) + d.off,
                         8 * (size_t)d.n, cudaMemcpyDeviceToDevice, c.stream));
  }
  CU(cudaStreamSynchronize(c.stream));
  return HF_OK;
}
int snapshot_restore(Ctx& c, const Snapshot& sn) {
  for (int64_t i = 0; i < c.ninst; ++i) {
    const InstDesc& d = c.h_inst[i];
    for (int k = 0; k < 4; ++k)
      CU(cudaMemcpyAsync(snapshot_field(c, sn.scal[i], k) + d.off, sn.t + k * c.ncells + d.off,
                         8 * (size_t)d.n, cudaMemcpyDeviceToDevice, c.stream));
  }
  std::memcpy(c.h_scal, sn.scal.data(), sizeof(InstScal) * c.ninst);
  return push_scal(c, true);
}
}  // namespace

extern "C" {

int hf_set_property_tables(hf_ctx* h, int32_t ntables, const int32_t* offsets, const double* rows,
                           const int32_t* cell_table) {
  if (!h || ntables < 0 || (ntables > 0 && (!offsets || !rows || !cell_table)))
    return set_err(HF_EARG, "bad arguments");
  Ctx& c = h->c;
  if (int r_ = refuse_queued(c)) return r_;
  if (ntables == 0) {                         // back to fixed properties
    c.tempdep = false;
    drop_graph(c);
    return HF_OK;
  }
  if (offsets[0] != 0) return set_err(HF_EARG, "offsets[0] must be 0");
  for (int32_t k = 0; k < ntables; ++k) {
    const int32_t m = offsets[k + 1] - offsets[k];
    if (m < 1) return set_err(HF_EARG, "every table needs at least one row");
    for (int32_t r = offsets[k]; r < offsets[k + 1]; ++r) {
      if (!(rows[4 * r + 1] > 0.0) || !(rows[4 * r + 2] > 0.0) || !(rows[4 * r + 3] > 0.0))
        return set_err(HF_EARG, "table kappa, rho and c must be positive");
      if (r > offsets[k] && !(rows[4 * r] > rows[4 * (r - 1)]))
        return set_err(HF_EARG, "table temperatures must increase");
    }
  }
  int64_t total = 0;
  for (int64_t i = 0; i < c.ninst; ++i) total += c.h_inst[i].n;
  std::vector<int32_t> ct((size_t)c.ncells, -1);
  {
    int64_t pos = 0;
    for (int64_t i = 0; i < c.ninst; ++i) {
      const InstDesc& d = c.h_inst[i];
      for (int64_t l = 0; l < d.n; ++l) {
        const int32_t t = cell_table[pos + l];
        if (t < -1 || t >= ntables) return set_err(HF_EARG, "cell table index out of range");
        ct[(size_t)(d.off + l)] = t;
      }
      pos += d.n;
    }
  }
  (void)total;
  if (!c.d_cell_table) {
    int r = dalloc(c, &c.d_cell_table, (size_t)c.ncells);
    if (r) return r;
  }
  for (void* p : {(void*)c.d_toff, (void*)c.d_trows}) {
    if (!p) continue;
    cudaFree(p);
    c.allocs.erase(std::remove(c.allocs.begin(), c.allocs.end(), p), c.allocs.end());
  }
  c.d_toff = nullptr;
  c.d_trows = nullptr;
  int r = dalloc(c, &c.d_toff, (size_t)ntables + 1);
  if (!r) r = dalloc(c, &c.d_trows, 4 * (size_t)offsets[ntables]);
  if (r) return r;
  CU(cudaMemcpy(c.d_toff, offsets, sizeof(int32_t) * ((size_t)ntables + 1), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(c.d_trows, rows, sizeof(double) * 4 * (size_t)offsets[ntables], cudaMemcpyHostToDevice));
  CU(cudaMemcpy(c.d_cell_table, ct.data(), sizeof(int32_t) * ct.size(), cudaMemcpyHostToDevice));
  c.tempdep = true;
  drop_graph(c);                              // the captured steps gain the rebuild kernels
  return HF_OK;
}

int hf_subbox_async(hf_ctx* h, int64_t inst, const int64_t* lo, const int64_t* hi, int which,
                    double* host, int64_t* ticket) {
  if (!h || !lo || !hi || !host || !ticket || (which != 0 && which != 1))
    return set_err(HF_EARG, "bad arguments");
  Ctx& c = h->c;
  if (int r_ = refuse_queued(c)) return r_;
  if (inst < 0 || inst >= c.ninst) return set_err(HF_EARG, "instance out of range");
  const InstDesc& d = c.h_inst[inst];
  const int64_t dims[3] = {d.nx, d.ny, d.nz};
  int64_t n = 1;
  for (int k = 0; k < 3; ++k) {
    if (lo[k] < 0 || hi[k] < lo[k] || hi[k] >= dims[k]) return set_err(HF_EARG, "box outside the grid");
    n *= hi[k] - lo[k] + 1;
  }
  if (!c.state_set) return set_err(HF_ESTATE, "hf_set_state must be called first");
  if (!c.copy_stream) CU(cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking));
  Ctx::SubSlot& sl = c.sub[c.next_ticket % Ctx::kSubSlots];
  if (!sl.gathered) {
    CU(cudaEventCreateWithFlags(&sl.gathered, cudaEventDisableTiming));
    CU(cudaEventCreateWithFlags(&sl.copied, cudaEventDisableTiming));
  }
  if (sl.cap < (size_t)n) {                    // grow the slot (after its previous copy)
    if (sl.dev) {
      CU(cudaEventSynchronize(sl.copied));
      CU(cudaFree(sl.dev));
      sl.dev = nullptr;
    }
    CU(cudaMalloc((void**)&sl.dev, sizeof(double) * (size_t)n));
    sl.cap = (size_t)n;
  } else if (sl.ticket >= 0) {
    CU(cudaStreamWaitEvent(c.stream, sl.copied, 0));   // the slot's previous copy has finished
  }
  CU(launch_subbox_gather(c, inst, lo, hi, which, sl.dev));
  CU(cudaEventRecord(sl.gathered, c.stream));
  CU(cudaStreamWaitEvent(c.copy_stream, sl.gathered, 0));
  CU(cudaMemcpyAsync(host, sl.dev, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, c.copy_stream));
  CU(cudaEventRecord(sl.copied, c.copy_stream));
  sl.ticket = c.next_ticket;
  *ticket = c.next_ticket++;
  c.launches += 1;
  return HF_OK;
}

int hf_subbox_wait(hf_ctx* h, int64_t ticket) {
  if (!h || ticket < 0) return set_err(HF_EARG, "bad arguments");
  Ctx& c = h->c;
  if (ticket >= c.next_ticket) return set_err(HF_EARG, "unknown ticket");
  // a slot's event covers its latest copy; copies on the copy stream complete in order, so a
  // reused slot's event also covers every earlier ticket of that slot
  Ctx::SubSlot& sl = c.sub[ticket % Ctx::kSubSlots];
  if (sl.copied) CU(cudaEventSynchronize(sl.copied));
  return HF_OK;
}

int hf_autotune(hf_ctx* h, int64_t itime0, int32_t steps, hf_tune_result* results, int32_t cap,
                int32_t* n_results) {
  if (!h || steps < 1 || cap < 0 || (cap > 0 && !results)) return set_err(HF_EARG, "bad arguments");
  Ctx& c = h->c;
  if (!c.state_set) return set_err(HF_ESTATE, "hf_set_state must be called first");
  Snapshot sn;
  int rc = snapshot_take(c, sn);
  if (rc) { cudaFree(sn.t); return rc; }
  const hf_solver_opts base = c.opts;
  const bool mixed = base.precision == HF_PREC_MIXED;
  const int depths[4] = {8, 16, 32, 64};
  const double tols[3] = {1e-4, 1e-5, 1e-6};
  const int ntol = mixed ? 3 : 1;
  std::vector<hf_tune_result> all;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  auto finish = [&](int code) {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(sn.t);
    return code;
  };
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return finish(set_err(HF_ECUDA, "cudaEventCreate failed"));
  for (int di = 0; di < 4; ++di) {
    for (int ti = 0; ti < ntol; ++ti) {
      hf_solver_opts o = base;
      o.task_depth = depths[di];
      if (mixed) o.inner_tol = tols[ti];
      if ((rc = hf_set_opts(h, &o))) return finish(rc);
      if ((rc = snapshot_restore(c, sn))) return finish(rc);
      if ((rc = run_steps(c, itime0, 1, nullptr))) return finish(rc);     // warm-up (and capture)
      if ((rc = snapshot_restore(c, sn))) return finish(rc);
      if (cudaEventRecord(e0, c.stream) != cudaSuccess) return finish(set_err(HF_ECUDA, "event"));
      if ((rc = run_steps(c, itime0, steps, nullptr))) return finish(rc);
      if (cudaEventRecord(e1, c.stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
        return finish(set_err(HF_ECUDA, "event"));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      all.push_back(hf_tune_result{depths[di], 0, o.inner_tol, (double)ms / steps});
    }
  }
  size_t best = 0;
  for (size_t k = 1; k < all.size(); ++k)
    if (all[k].ms_per_step < all[best].ms_per_step) best = k;
  all[best].chosen = 1;
  hf_solver_opts o = base;
  o.task_depth = all[best].task_depth;
  if (mixed) o.inner_tol = all[best].inner_tol;
  if ((rc = hf_set_opts(h, &o))) return finish(rc);
  if ((rc = snapshot_restore(c, sn))) return finish(rc);
  if (n_results) *n_results = (int32_t)std::min<size_t>(all.size(), (size_t)cap);
  for (size_t k = 0; k < all.size() && (int32_t)k < cap; ++k) results[k] = all[k];
  return finish(HF_OK);
}

}  // extern "C"

namespace {
// Time the persistent solve alone: each repetition begins the next step and forms its RHS
// (untimed), then times one solve with CUDA events on the context stream.  T^n and T^(n-1) are
// not modified (the step's end, which rotates them, does not run); the scalars are restored.
// A copy of every instance's H T^(n-1) (the product slot a solve's last sweep overwrites), for the
// calls that run solves outside the step sequence and then give the context back unchanged.
struct HxKeep {
  Ctx& c;
  const std::vector<InstScal>& scal;
  double* buf = nullptr;
  HxKeep(Ctx& ctx, const std::vector<InstScal>& s) : c(ctx), scal(s) {}
  ~HxKeep() { if (buf) cudaFree(buf); }
  double* slot(int64_t i) const { return c.A.hx[1 - scal[i].hx_role] + c.h_inst[i].off; }
  cudaError_t copy(bool save) {
    for (int64_t i = 0; i < c.ninst; ++i) {
      const int64_t off = c.h_inst[i].off, n = c.h_inst[i].n;
      cudaError_t e = save ? cudaMemcpyAsync(buf + off, slot(i), 8 * n, cudaMemcpyDeviceToDevice, c.stream)
                           : cudaMemcpyAsync(slot(i), buf + off, 8 * n, cudaMemcpyDeviceToDevice, c.stream);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  int save() {
    cudaError_t e = cudaMalloc(&buf, sizeof(double) * (size_t)c.ncells);
    if (e == cudaSuccess) e = copy(true);
    return e == cudaSuccess ? HF_OK : set_err(HF_ECUDA, std::string("H T copy: ") + cudaGetErrorString(e));
  }
};

int time_solve(Ctx& c, int reps, double* ms) {
  if (!c.state_set) return set_err(HF_ESTATE, "hf_set_state must be called first");
  int rc = sync_scal(c);
  if (rc) return rc;
  std::vector<InstScal> saved(c.h_scal, c.h_scal + c.ninst);
  const int64_t itime = saved[0].itime + 1;
  // each solve's last sweep overwrites H T^(n-1), which the next repetition's first residual
  // reads: put it back before every repetition (outside the timed region)
  HxKeep keep(c, saved);
  if ((rc = keep.save())) return rc;
  cudaEvent_t e0, e1;
  CU(cudaEventCreate(&e0));
  CU(cudaEventCreate(&e1));
  double total = 0.0;
  for (int r = 0; r < reps; ++r) {
    CU(keep.copy(false));
    CU(launch_step_begin(c, itime, 0));
    CU(launch_rhs(c));
    CU(launch_finalize(c, FIN_RHS, nullptr, 0, 0));
    CU(cudaEventRecord(e0, c.stream));
    CU(launch_solve(c));
    CU(cudaEventRecord(e1, c.stream));
    CU(cudaEventSynchronize(e1));
    float t = 0.f;
    CU(cudaEventElapsedTime(&t, e0, e1));
    total += t;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CU(keep.copy(false));
  CU(cudaStreamSynchronize(c.stream));
  SolveCtl sc;
  CU(cudaMemcpy(&sc, c.d_sctl, sizeof(sc), cudaMemcpyDeviceToHost));
  std::memcpy(c.h_scal, saved.data(), sizeof(InstScal) * c.ninst);
  if ((rc = push_scal(c, true))) return rc;
  if (sc.err) return set_err(HF_EDEVICE, "persistent solve: a grid barrier wait reached its time limit");
  if (sc.guard_hit) return set_err(HF_EDEVICE, "persistent solve reached its round bound");
  *ms = total / reps;
  return HF_OK;
}
}  // namespace

extern "C" {

int hf_check_barrier_timeout(hf_ctx* h, int32_t wait_ms, int32_t* status, double* seconds) {
  if (!h || !status || wait_ms < 1 || wait_ms > 10000) return set_err(HF_EARG, "bad arguments");
  Ctx& c = h->c;
  if (!c.state_set) return set_err(HF_ESTATE, "hf_set_state must be called first");
  if (solve_grid_blocks(c, c.opts.precision == HF_PREC_MIXED ? 1 : 0) < 2)
    return set_err(HF_EARG, "the check needs a grid of at least two blocks");
  int rc = sync_scal(c);
  if (rc) return rc;
  std::vector<InstScal> saved(c.h_scal, c.h_scal + c.ninst);
  HxKeep keep(c, saved);                 // the abandoned solve may have written H T^(n-1)
  if ((rc = keep.save())) return rc;
  CU(launch_step_begin(c, saved[0].itime + 1, 0));
  CU(launch_rhs(c));
  CU(launch_finalize(c, FIN_RHS, nullptr, 0, 0));
  cudaEvent_t e0, e1;
  CU(cudaEventCreate(&e0));
  CU(cudaEventCreate(&e1));
  CU(cudaEventRecord(e0, c.stream));
  CU(launch_solve(c, (unsigned long long)wait_ms * 1000000ull, 0));
  CU(cudaEventRecord(e1, c.stream));
  CU(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  SolveCtl sc;
  CU(cudaMemcpy(&sc, c.d_sctl, sizeof(sc), cudaMemcpyDeviceToHost));
  *status = sc.err ? HF_EDEVICE : (sc.guard_hit ? HF_EDEVICE : HF_OK);
  if (seconds) *seconds = ms * 1e-3;
  CU(keep.copy(false));
  std::memcpy(c.h_scal, saved.data(), sizeof(InstScal) * c.ninst);
  return push_scal(c, true);
}

int hf_step_timeline(hf_ctx* h, double* us) {
  if (!h || !us) return set_err(HF_EARG, "null argument");
  Ctx& c = h->c;
  if (int r_ = refuse_queued(c)) return r_;
  unsigned long long t[kStamps];
  CU(cudaStreamSynchronize(c.stream));
  CU(cudaMemcpy(t, c.A.stamps, sizeof(t), cudaMemcpyDeviceToHost));
  // intervals between consecutive stamps; -1 where a stamp of the chain was not written in order
  for (int k = 0; k < 5; ++k) {
    const unsigned long long a = t[k], b = t[k + 1];
    us[k] = (a != 0 && b >= a) ? (double)(b - a) * 1e-3 : -1.0;
  }
  return HF_OK;
}

int hf_solve_profile(hf_ctx* h, int64_t cap, int64_t* rounds, int32_t* phases, double* round_us) {
  if (!h || !rounds || cap < 0 || (cap > 0 && (!phases || !round_us)))
    return set_err(HF_EARG, "bad arguments");
  Ctx& c = h->c;
  if (int r_ = refuse_queued(c)) return r_;
  SolveCtl sc;
  CU(cudaStreamSynchronize(c.stream));
  CU(cudaMemcpy(&sc, c.d_sctl, sizeof(sc), cudaMemcpyDeviceToHost));
  *rounds = sc.rounds;
  const int64_t n = std::min<int64_t>(std::min<int64_t>(sc.rounds, cap), kRoundLog);
  unsigned long long prev = sc.t_start;
  for (int64_t r = 0; r < n; ++r) {
    phases[r] = sc.phase_log[r];
    round_us[r] = (double)(sc.t_round[r] - prev) * 1e-3;
    prev = sc.t_round[r];
  }
  return HF_OK;
}

int hf_index_checks(hf_ctx* h, int32_t probe, int32_t* enabled, int64_t* record) {
  if (!h || !enabled) return set_err(HF_EARG, "null argument");
  Ctx& c = h->c;
  if (int r = refuse_queued(c)) return r;
#ifdef HF_CHECKED
  *enabled = 1;
  if (probe) {
    CU(launch_check_probe(c));
    CU(cudaStreamSynchronize(c.stream));
  }
#else
  *enabled = 0;
  (void)probe;
#endif
  unsigned long long rec[4] = {0, 0, 0, 0};
  CU(cudaMemcpyAsync(rec, c.A.check, sizeof(rec), cudaMemcpyDeviceToHost, c.stream));
  CU(cudaMemsetAsync(c.A.check, 0, sizeof(rec), c.stream));
  CU(cudaStreamSynchronize(c.stream));
  if (record)
    for (int k = 0; k < 4; ++k) record[k] = (int64_t)rec[k];
  return HF_OK;
}

int hf_time_kernel(hf_ctx* h, int which, int reps, double* ms) {
  if (!h || !ms || reps < 1 || which < HF_KERNEL_RHS || which > HF_KERNEL_RESIDUAL_INIT)
    return set_err(HF_EARG, "bad arguments");
  if (which == HF_KERNEL_SOLVE) return time_solve(h->c, reps, ms);
  Ctx& c = h->c;
  if (!c.state_set) return set_err(HF_ESTATE, "hf_set_state must be called first");
  int rc = sync_scal(c);
  if (rc) return rc;
  std::vector<InstScal> saved(c.h_scal, c.h_scal + c.ninst);
  std::vector<InstScal> phase = saved;
  for (auto& s : phase) {
    s.outer_active = 1;
    const bool cg = (which >= HF_KERNEL_CG_P && which <= HF_KERNEL_CG_UPDATE) || which == HF_KERNEL_CG_PQ;
    s.inner_active = cg ? 1 : 0;
    s.refine = which == HF_KERNEL_RESIDUAL_INIT ? 0 : 1;
    s.iter = (which == HF_KERNEL_CG_P || which == HF_KERNEL_CG_UPDATE || which == HF_KERNEL_CG_PQ ||
              which == HF_KERNEL_RESIDUAL) ? 1 : 0;
    s.status = 0;
    s.rho = 1.0; s.gg0 = 1.0; s.beta = 0.5; s.alpha = 0.5; s.eta = 0.0;
    s.sigma = 1.0; s.sigma_prev = 1.0;
    s.xw = 0;                     // the plain CG update and x update
    if (s.bb <= 0.0) s.bb = 1.0;
  }
  cudaEvent_t e0, e1;
  CU(cudaEventCreate(&e0));
  CU(cudaEventCreate(&e1));
  double total = 0.0;
  for (int r = 0; r < reps; ++r) {
    std::memcpy(c.h_scal, phase.data(), sizeof(InstScal) * c.ninst);
    CU(cudaMemcpyAsync(c.A.scal, c.h_scal, sizeof(InstScal) * c.ninst, cudaMemcpyHostToDevice, c.stream));
    CU(cudaEventRecord(e0, c.stream));
    CU(launch_single(c, which));
    CU(cudaEventRecord(e1, c.stream));
    CU(cudaEventSynchronize(e1));
    float t = 0.f;
    CU(cudaEventElapsedTime(&t, e0, e1));
    total += t;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  std::memcpy(c.h_scal, saved.data(), sizeof(InstScal) * c.ninst);
  // only the residual sweep after an update writes the stored products H T
  if ((rc = push_scal(c, which != HF_KERNEL_RESIDUAL))) return rc;
  *ms = total / reps;
  return HF_OK;
}

int hf_get_operator(hf_ctx* h, double* diag, double* cx, double* cy, double* cz) {
  if (!h) return set_err(HF_EARG, "null context");
  Ctx& c = h->c;
  if (int r_ = refuse_queued(c)) return r_;
  int rc;
  if (diag && (rc = download_padded(c, diag, c.A.diag))) return rc;
  if (cx && (rc = download_padded(c, cx, c.A.cx))) return rc;
  if (cy && (rc = download_padded(c, cy, c.A.cy))) return rc;
  if (cz && (rc = download_padded(c, cz, c.A.cz))) return rc;
  CU(cudaStreamSynchronize(c.stream));
  return HF_OK;
}

int hf_apply_operator(hf_ctx* h, const double* x, double* y) {
  if (!h || !x || !y) return set_err(HF_EARG, "null argument");
  Ctx& c = h->c;
  if (int r_ = refuse_queued(c)) return r_;
  int rc;
  if ((rc = upload_padded(c, c.A.p, x))) return rc;   // p and q are free outside a step
  CU(launch_apply(c, c.A.p, c.A.q));
  if ((rc = download_padded(c, y, c.A.q))) return rc;
  CU(cudaStreamSynchronize(c.stream));
  return HF_OK;
}

int hf_get_rhs(hf_ctx* h, int64_t itime, double* B, double* Q, double* Qd, double* sc, double* S,
               double* x0) {
  if (!h) return set_err(HF_EARG, "null context");
  Ctx& c = h->c;
  if (!c.state_set) return set_err(HF_ESTATE, "hf_set_state must be called first");
  // scratch: the FP64 CG vectors are free outside a step
  CU(launch_step_begin(c, itime, 0));
  CU(launch_rhs_parts(c, c.A.y, c.A.r, c.A.p, c.A.q));
  CU(launch_finalize(c, FIN_RHS, nullptr, 0, 0));
  int rc = sync_scal(c);
  if (rc) return rc;
  if ((rc = diagnose(c))) return rc;
  if (B && (rc = download_padded(c, B, (const double*)c.A.y))) return rc;
  if (Q && (rc = download_padded(c, Q, (const double*)c.A.r))) return rc;
  if (Qd && (rc = download_padded(c, Qd, (const double*)c.A.p))) return rc;
  if (sc && (rc = download_padded(c, sc, (const double*)c.A.q))) return rc;
  if (S && (rc = download_padded(c, S, (const double*)c.A.b))) return rc;
  int64_t pos = 0;
  for (int64_t i = 0; i < c.ninst; ++i) {
    const InstDesc& d = c.h_inst[i];
    const InstScal& s = c.h_scal[i];
    if (x0) CU(cudaMemcpyAsync(x0 + pos, c.A.tbuf[s.role[2]] + d.off, 8 * d.n, cudaMemcpyDeviceToHost, c.stream));
    pos += d.n;
  }
  CU(cudaStreamSynchronize(c.stream));
  if (x0) {
    pos = 0;
    for (int64_t i = 0; i < c.ninst; ++i) {
      const InstDesc& d = c.h_inst[i];
      if (c.h_scal[i].x0flag)
        for (int64_t k = 0; k < d.n; ++k) x0[pos + k] = x0[pos + k] + kTiny;   // mod_evolve.f90:141
      pos += d.n;
    }
  }
  for (int64_t i = 0; i < c.ninst; ++i)
    if (c.h_scal[i].status) return status_code(c.h_scal[i].status);
  return HF_OK;
}

}  // extern "C"

namespace {
// The solve of hf_solve / hf_solve_device after the scalars were set up: one persistent launch
// (use_graph = 1) or the host-polled kernels.
int device_solve(Ctx& c) {
  if (c.opts.use_graph == 1 || c.opts.use_graph == 3) {
    if (solve_grid_blocks(c, c.opts.precision == HF_PREC_MIXED ? 1 : 0) < 1)
      return set_err(HF_ECUDA, "no co-resident grid for the persistent solve kernel");
    CU(launch_solve(c));
    SolveCtl sc;
    CU(cudaMemcpyAsync(&sc, c.d_sctl, sizeof(sc), cudaMemcpyDeviceToHost, c.stream));
    CU(cudaStreamSynchronize(c.stream));
    c.launches += 1;
    if (sc.err) return set_err(HF_EDEVICE, "persistent solve: a grid barrier wait reached its time limit");
    if (sc.guard_hit) return set_err(HF_EDEVICE, "persistent solve reached its round bound");
    return HF_OK;
  }
  CU(launch_residual(c, 0));
  return solve_loop(c);
}
}  // namespace

extern "C" {

int hf_solve(hf_ctx* h, const double* b, double* x, hf_stats* stats) {
  if (!h || !b || !x) return set_err(HF_EARG, "null argument");
  Ctx& c = h->c;
  if (c.ninst != 1) return set_err(HF_EARG, "hf_solve takes single-grid contexts");
  int rc = sync_scal(c);
  if (rc) return rc;
  std::vector<InstScal> before(c.h_scal, c.h_scal + 1);
  const InstDesc& d = c.h_inst[0];
  InstScal& s = c.h_scal[0];
  double bb = 0.0;
  for (int64_t k = 0; k < d.n; ++k) bb += b[k] * b[k];
  CU(cudaMemcpyAsync(c.A.b + d.off, b, 8 * d.n, cudaMemcpyHostToDevice, c.stream));
  CU(cudaMemcpyAsync(c.A.tbuf[s.role[2]] + d.off, x, 8 * d.n, cudaMemcpyHostToDevice, c.stream));
  s.bb = bb;
  s.itime = 0;
  s.outer_active = 1;
  s.inner_active = 0;
  s.refine = 0;
  s.iter = 0;
  s.step_iters = 0;
  s.x0flag = 0;
  s.status = 0;
  double rms = std::sqrt(bb / (double)d.n) * d.mean_sinv * 1e-6;
  s.sigma = (c.opts.precision == HF_PREC_MIXED && rms > 0.0 && std::isfinite(rms))
                ? std::exp2(std::rint(std::log2(rms))) : 1.0;
  s.xw = 0;
  s.phase = PH_RES_INIT;
  if ((rc = push_scal(c))) return rc;
  if ((rc = device_solve(c))) return rc;
  if ((rc = sync_scal(c))) return rc;
  CU(cudaMemcpyAsync(x, c.A.tbuf[c.h_scal[0].role[2]] + d.off, 8 * d.n, cudaMemcpyDeviceToHost, c.stream));
  CU(cudaStreamSynchronize(c.stream));
  fill_stats(c, stats, 0, before);
  return first_error(c);
}

int hf_set_state_device(hf_ctx* h, const double* tp, const double* tpp) {
  if (!h || !tp || !tpp) return set_err(HF_EARG, "null argument");
  Ctx& c = h->c;
  if (c.ninst != 1) return set_err(HF_EARG, "device state transfer takes single-grid contexts");
  int rc = sync_scal(c);
  if (rc) return rc;
  const InstDesc& d = c.h_inst[0];
  const InstScal& s = c.h_scal[0];
  CU(cudaMemcpyAsync(c.A.tbuf[s.role[0]] + d.off, tp, 8 * d.n, cudaMemcpyDeviceToDevice, c.stream));
  CU(cudaMemcpyAsync(c.A.tbuf[s.role[1]] + d.off, tpp, 8 * d.n, cudaMemcpyDeviceToDevice, c.stream));
  c.state_set = true;
  return push_scal(c);   // a new state: the stored products H T are stale
}

int hf_get_state_device(hf_ctx* h, double* tp, double* tpp) {
  if (!h) return set_err(HF_EARG, "null context");
  Ctx& c = h->c;
  if (c.ninst != 1) return set_err(HF_EARG, "device state transfer takes single-grid contexts");
  int rc = sync_scal(c);
  if (rc) return rc;
  const InstDesc& d = c.h_inst[0];
  const InstScal& s = c.h_scal[0];
  if (tp) CU(cudaMemcpyAsync(tp, c.A.tbuf[s.role[0]] + d.off, 8 * d.n, cudaMemcpyDeviceToDevice, c.stream));
  if (tpp) CU(cudaMemcpyAsync(tpp, c.A.tbuf[s.role[1]] + d.off, 8 * d.n, cudaMemcpyDeviceToDevice, c.stream));
  CU(cudaStreamSynchronize(c.stream));
  return HF_OK;
}

int hf_solve_device(hf_ctx* h, const double* b, double* x, hf_stats* stats) {
  if (!h || !b || !x) return set_err(HF_EARG, "null argument");
  Ctx& c = h->c;
  if (c.ninst != 1) return set_err(HF_EARG, "hf_solve_device takes single-grid contexts");
  int rc = sync_scal(c);
  if (rc) return rc;
  std::vector<InstScal> before(c.h_scal, c.h_scal + 1);
  const InstDesc& d = c.h_inst[0];
  InstScal& s = c.h_scal[0];
  s.itime = 0;
  s.outer_active = 1;
  s.inner_active = 0;
  s.refine = 0;
  s.iter = 0;
  s.step_iters = 0;
  s.x0flag = 0;
  s.tiny_pending = 0;
  s.status = 0;
  s.xw = 0;
  s.phase = PH_RES_INIT;
  if ((rc = push_scal(c))) return rc;
  CU(cudaMemcpyAsync(c.A.b + d.off, b, 8 * d.n, cudaMemcpyDeviceToDevice, c.stream));
  CU(cudaMemcpyAsync(c.A.tbuf[s.role[2]] + d.off, x, 8 * d.n, cudaMemcpyDeviceToDevice, c.stream));
  CU(launch_sumsq(c, c.A.b + d.off, d.n));
  if ((rc = device_solve(c))) return rc;
  if ((rc = sync_scal(c))) return rc;
  CU(cudaMemcpyAsync(x, c.A.tbuf[c.h_scal[0].role[2]] + d.off, 8 * d.n, cudaMemcpyDeviceToDevice, c.stream));
  CU(cudaStreamSynchronize(c.stream));
  fill_stats(c, stats, 0, before);
  return first_error(c);
}

int hf_adjoint_rhs(hf_ctx* h, const double* g, const double* l1, const double* l2, double* out) {
  if (!h || !g || !l1 || !l2 || !out) return set_err(HF_EARG, "null argument");
  Ctx& c = h->c;
  if (int r_ = refuse_queued(c)) return r_;
  if (c.ninst != 1) return set_err(HF_EARG, "the adjoint takes single-grid contexts");
  CU(launch_adj_rhs(c, g, l1, l2, out));
  CU(cudaStreamSynchronize(c.stream));
  return HF_OK;
}

int hf_adjoint_accumulate(hf_ctx* h, const double* lam, const double* x, int64_t itime,
                          double* grad_logk, double* grad_src) {
  if (!h || !lam || !x || !grad_logk) return set_err(HF_EARG, "null argument");
  Ctx& c = h->c;
  if (int r_ = refuse_queued(c)) return r_;
  if (c.ninst != 1) return set_err(HF_EARG, "the adjoint takes single-grid contexts");
  for (int f = 0; f < 6; ++f)
    if (c.h_bc[0].cg[f]) return set_err(HF_EARG, "the adjoint does not differentiate Neumann (CG) faces");
  if (c.h_inst[0].has_em) return set_err(HF_EARG, "the adjoint does not differentiate the radiative term");
  CU(launch_adj_grad(c, lam, x, itime, grad_logk, grad_src));
  CU(cudaStreamSynchronize(c.stream));
  return HF_OK;
}

int hf_assemble_coo(hf_ctx* h, int64_t inst, int64_t cap, int64_t* irow, int64_t* jcol, double* val,
                    int64_t* len, int64_t* count) {
  if (!h) return set_err(HF_EARG, "null context");
  Ctx& c = h->c;
  if (int r_ = refuse_queued(c)) return r_;
  if (inst < 0 || inst >= c.ninst) return set_err(HF_EARG, "instance out of range");
  const InstDesc& d = c.h_inst[inst];
  const int64_t nx = d.nx, ny = d.ny, nz = d.nz;
  int64_t L = 7 * nx * ny * nz - 2 * (nx * ny + ny * nz + nz * nx);   // mod_setup.f90:96-99
  if (d.px) L += 2 * ny * nz;
  if (d.py) L += 2 * nz * nx;
  if (d.pz) L += 2 * nx * ny;
  if (len) *len = L;
  if (!irow || !jcol || !val) return HF_OK;
  if (cap < L) return set_err(HF_EARG, "capacity below the reference's COO length");
  int64_t *d_counts = nullptr, *d_pos = nullptr, *d_irow = nullptr, *d_jcol = nullptr;
  double* d_val = nullptr;
  auto cleanup = [&]() { cudaFree(d_counts); cudaFree(d_pos); cudaFree(d_irow); cudaFree(d_jcol); cudaFree(d_val); };
  if (cudaMalloc(&d_counts, 8 * d.n) != cudaSuccess || cudaMalloc(&d_pos, 8 * d.n) != cudaSuccess ||
      cudaMalloc(&d_irow, 8 * std::max<int64_t>(L, 1)) != cudaSuccess ||
      cudaMalloc(&d_jcol, 8 * std::max<int64_t>(L, 1)) != cudaSuccess ||
      cudaMalloc(&d_val, 8 * std::max<int64_t>(L, 1)) != cudaSuccess) {
    cleanup();
    return set_err(HF_ENOMEM, "COO scratch allocation failed");
  }
  std::vector<int64_t> counts((size_t)d.n), pos((size_t)d.n);
  cudaError_t e = launch_coo(c, inst, d_counts, nullptr, nullptr, nullptr, nullptr, 0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(counts.data(), d_counts, 8 * d.n, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) { cleanup(); return set_err(HF_ECUDA, cudaGetErrorString(e)); }
  int64_t run = 0;
  for (int64_t k = 0; k < d.n; ++k) { pos[k] = run; run += counts[k]; }
  if (run > L) { cleanup(); return set_err(HF_EARG, "entries exceed the reference's COO capacity"); }
  std::vector<int64_t> hi((size_t)L, -2), hj((size_t)L, -1);
  std::vector<double> hv((size_t)L, 0.0);
  e = cudaMemcpyAsync(d_pos, pos.data(), 8 * d.n, cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess && L > 0) e = cudaMemcpyAsync(d_irow, hi.data(), 8 * L, cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess && L > 0) e = cudaMemcpyAsync(d_jcol, hj.data(), 8 * L, cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess && L > 0) e = cudaMemcpyAsync(d_val, hv.data(), 8 * L, cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess) e = launch_coo(c, inst, nullptr, d_irow, d_jcol, d_val, d_pos, 1);
  if (e == cudaSuccess && L > 0) e = cudaMemcpyAsync(irow, d_irow, 8 * L, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess && L > 0) e = cudaMemcpyAsync(jcol, d_jcol, 8 * L, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess && L > 0) e = cudaMemcpyAsync(val, d_val, 8 * L, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  cleanup();
  if (e != cudaSuccess) return set_err(HF_ECUDA, cudaGetErrorString(e));
  if (count) *count = run;
  return HF_OK;
}

}  // extern "C"
