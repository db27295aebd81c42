// Host-side context of libheatflow_gb300 (one or more grids on one GPU).
#pragma once

#include <string>
#include <vector>

#include "hf_internal.cuh"

namespace hf {

// Assembly-only device inputs (kept for the parity probes, not read per step).
struct AsmArrays {
  double *kappa = nullptr, *tau_s = nullptr;
  // per instance: boundary-condition block
};

struct InstBC {
  double kb[6], tb[6], pd[6], br;
  int32_t cg[6];
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int64_t ninst = 0, ncells = 0, ntiles = 0;
  int64_t ntasks = 0;            // blocks of the step kernels
  int64_t ntasks_cap = 0;        // task buffers' capacity (shallowest task depth)
  int depth = 0;                 // task depth of the current table
  std::vector<InstDesc> h_inst;
  std::vector<InstBC> h_bc;
  std::vector<int64_t> h_tile0;
  hf_solver_opts opts{};
  DevArrays A{};
  AsmArrays asm_{};
  InstBC* d_bc = nullptr;
  std::vector<void*> allocs;
  InstScal* h_scal = nullptr;    // pinned mirror for polling
  bool state_set = false;
  bool any_heater = false, any_power = false, any_em = false, any_case5 = false;
  // graph of one step (hf_run replays it once per step, no host synchronisation in between)
  cudaGraphExec_t graph_exec = nullptr;
  cudaGraph_t graph = nullptr;
  CtrlState* d_ctrl = nullptr;
  SolveCtl* d_sctl = nullptr;    // control block of the persistent solve kernel
  int solve_blocks[2] = {0, 0};  // co-resident grid of the persistent solve (FP64, FP32)
  int graph_mode = 0;            // use_graph value the graph was captured for
  // use_graph = 1: the whole time loop as one graph (WHILE node around one step)
  cudaGraphExec_t loop_exec = nullptr;
  cudaGraph_t loop_graph = nullptr;
  bool loop_unsupported = false;  // capture or instantiation refused: per-step graphs instead
  int graph_precision = -1;     // options the graph was captured with
  int graph_criterion = -1;
  int64_t launches = 0;          // kernels launched on the device since creation
  // sub-box snapshots: staging slots copied to the host on a second stream
  struct SubSlot {
    double* dev = nullptr;
    size_t cap = 0;                // doubles
    cudaEvent_t gathered = nullptr, copied = nullptr;
    int64_t ticket = -1;
  };
  static constexpr int kSubSlots = 4;
  SubSlot sub[kSubSlots];
  cudaStream_t copy_stream = nullptr;
  int64_t next_ticket = 0;
  // host-buffer steps queued without host round trips (hf_step_host_async): copy engines move
  // compact staging buffers; kernels place them into (and gather from) the role buffers
  static constexpr int kHostChunks = 8;
  static constexpr int kHostOuts = 4;
  // Downloads of the last kHostOuts queued steps (older ones are complete once a staging set's
  // free event has passed): the host array each writes, with events for the whole download and
  // chunk by chunk.  An upload from one of these arrays waits for its download, whatever order
  // the caller passes the arrays in.
  struct HostOut {
    const double* ptr = nullptr;
    cudaEvent_t done = nullptr;
    cudaEvent_t chunk[kHostChunks] = {};
  };
  HostOut outs[kHostOuts];
  int out_last = 0;                    // outs[out_last]: the last queued download
  // Two staging sets for the uploaded inputs, used by alternate calls, so a call's uploads need
  // not wait for the previous call's inputs to be consumed.
  struct Stage {
    double* p = nullptr;               // T^n of the call (compact layout)
    double* pp = nullptr;              // T^(n-1)
    cudaEvent_t in_pp = nullptr;       // T^(n-1) has landed
    cudaEvent_t in_chunk[kHostChunks] = {};   // ... T^n, chunk by chunk
    cudaEvent_t free = nullptr;        // the set's consumer (placement or check) has run
  };
  Stage stage[2];
  // The queued steps' results in the compact layout, written by each step's last residual sweep
  // (or, for a step accepted at its first residual, by the fallback copy after it), for alternate
  // calls; free again once the download that read it has run.
  double* d_stage_x[2] = {nullptr, nullptr};
  cudaEvent_t stage_x_free[2] = {nullptr, nullptr};
  // The queued calls.  A call whose inputs are the previous call's result and inputs (the
  // rotation simulate() performs) starts from the device's own copy of them ("early"), while its
  // uploads travel; the next call (or hf_host_sync) checks the uploaded bits against that copy.
  struct HostCall {
    int64_t itime;
    const double* tp;
    const double* tpp;
    double* out;
    bool early;
  };
  std::vector<HostCall> async_calls;
  int64_t* d_check_call = nullptr;     // first call whose uploads differed from the device copy
  int64_t async_host_kernels = 0;      // host-copy kernels of the queued calls
  // T^n moves in chunks of whole task z-slabs: each chunk's RHS tasks run as soon as its cells
  // are placed, while later chunks are still on the link.  Cells [clo, chi) of the compact host
  // layout, [glo, ghi) of the device layout, tasks [tlo, thi).
  struct HostChunk { int64_t clo, chi, glo, ghi, tlo, thi; };
  std::vector<HostChunk> host_chunks;
  int host_chunks_depth = -1;           // task depth the chunks were cut for
  cudaStream_t out_stream = nullptr;    // downloads, so the next step's work need not queue behind them
  cudaEvent_t ev_gathered = nullptr;    // the last queued step's result is in its d_stage_x
  // the step after its RHS (finalize, persistent solve, step end, result fallback, property
  // rebuild) as one graph per result buffer d_stage_x[j]
  cudaGraphExec_t post_exec[2] = {nullptr, nullptr};
  cudaGraph_t post_graph[2] = {nullptr, nullptr};
  int post_precision = -1, post_criterion = -1;
  bool async_pending = false;          // steps queued since the last hf_host_sync
  int64_t async_steps = 0;             // = async_calls.size()
  std::vector<InstScal> async_before;  // scalars before the first queued step
  // tabulated properties re-evaluated after every step (hf_set_property_tables)
  bool tempdep = false;
  int32_t* d_toff = nullptr;
  double* d_trows = nullptr;
  int32_t* d_cell_table = nullptr;
};

}  // namespace hf
