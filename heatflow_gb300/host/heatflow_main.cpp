// HeatFlow's main program on libheatflow_gb300 (src/heatflow.f90): read the deck, set up, run
// ntime steps, log the sub-box after step 1 and every write_every steps, and print the final
// fields.  The reference's file layout is kept: ./inputs/{param,mat,system}.in,
// ./restart/TempDis.dat[TPD] (initial_evolve, mod_init_evolve.f90:34-51),
// ./outputs/output_<RunName>_NN (data_write, mod_output.f90:57-113) and
// ./outputs/TempDis.dat[TPD] (final_print, mod_output.f90:207-238).
//
//   heatflow_gb300 [--inputs DIR] [--outputs DIR] [--restart DIR]
//                  [--precision fp64|mixed] [--criterion recursive|true] [--tol X]
//                  [--graph 0|1|2|3] [--dump-problem] [--dump-log-schedule]
//
// Defaults follow the reference: FP64 with linbcg's stopping rule (recursive residual, tol 1e-32),
// the whole step loop as CUDA graphs.  --dump-problem prints the parsed deck as JSON and stops
// before any GPU call; --dump-log-schedule prints, as JSON, the steps after which the sub-box log
// gets records and how many ([itime, records] pairs), and stops before any GPU call too.  A fatal condition prints the reference's message and exits with status 1
// (`stop 1`).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "deck.hpp"
#include "heatflow_gb300.h"

namespace {

struct Options {
  std::string inputs = "./inputs", outputs = "./outputs", restart = "./restart";
  int precision = HF_PREC_FP64, criterion = HF_STOP_RECURSIVE, use_graph = 1;
  double tol = -1.0;
  bool dump_problem = false, dump_log_schedule = false;
};

[[noreturn]] void usage(const char* msg) {
  std::fprintf(stderr, "%s\nusage: heatflow_gb300 [--inputs DIR] [--outputs DIR] [--restart DIR] "
                       "[--precision fp64|mixed] [--criterion recursive|true] [--tol X] "
                       "[--graph 0|1|2|3] [--dump-problem] [--dump-log-schedule]\n", msg);
  std::exit(2);
}

Options parse_args(int argc, char** argv) {
  Options o;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) usage(("missing value after " + a).c_str());
      return argv[++i];
    };
    if (a == "--inputs") o.inputs = next();
    else if (a == "--outputs") o.outputs = next();
    else if (a == "--restart") o.restart = next();
    else if (a == "--precision") {
      const std::string v = next();
      if (v == "fp64") o.precision = HF_PREC_FP64;
      else if (v == "mixed") o.precision = HF_PREC_MIXED;
      else usage("--precision takes fp64 or mixed");
    } else if (a == "--criterion") {
      const std::string v = next();
      if (v == "recursive") o.criterion = HF_STOP_RECURSIVE;
      else if (v == "true") o.criterion = HF_STOP_TRUE;
      else usage("--criterion takes recursive or true");
    } else if (a == "--tol") o.tol = std::atof(next().c_str());
    else if (a == "--graph") o.use_graph = std::atoi(next().c_str());
    else if (a == "--dump-problem") o.dump_problem = true;
    else if (a == "--dump-log-schedule") o.dump_log_schedule = true;
    else usage(("unknown argument " + a).c_str());
  }
  return o;
}

int fail_lib(int rc, const char* where) {
  const char* m = hf_strerror(rc);
  std::fprintf(stdout, " %s\n", m ? m : "");
  std::fprintf(stderr, "%s: %s\n", where, hf_last_error());
  return 1;
}

bool write_file(const std::string& path, const std::string& text) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  const bool ok = std::fwrite(text.data(), 1, text.size(), f) == text.size();
  return std::fclose(f) == 0 && ok;
}

}  // namespace

int main(int argc, char** argv) {
  const auto t0 = std::chrono::steady_clock::now();
  const Options opt = parse_args(argc, argv);
  std::printf(" Setup initialising\n");
  hfhost::Deck deck;
  try {
    const std::string param = hfhost::read_text_file(opt.inputs + "/param.in", "Error cannot find file: param.in");
    const std::string mat = hfhost::read_text_file(opt.inputs + "/mat.in", "Error cannot find file: mat.in");
    const std::string sys = hfhost::read_text_file(opt.inputs + "/system.in", "Error cannot find file: system.in");
    hfhost::build_deck(deck, param, mat, sys);
    // TempDepProp = 1: ChangeProp's per-material tables (mod_tempdep.f90:44-55), re-evaluated
    // after every step (mod_evolve.f90:172-174)
    if (deck.param.temp_dep_prop == 1) deck.tables = hfhost::load_material_tables(opt.inputs, deck.sys);
  } catch (const hfhost::InputError& e) {
    std::printf(" %s\n", e.what());
    return 1;
  }
  if (opt.dump_problem) {
    std::printf("%s\n", hfhost::problem_json(deck).c_str());
    return 0;
  }
  const hfhost::Param& P = deck.param;
  const int64_t n = deck.ncells();
  if (opt.dump_log_schedule) {
    std::printf("[");
    const char* sep = "";
    for (int64_t it = 1; it <= P.ntime; ++it) {
      const int k = hfhost::records_after(P, it);
      if (k > 0) {
        std::printf("%s[%lld, %d]", sep, (long long)it, k);
        sep = ", ";
      }
    }
    std::printf("]\n");
    return 0;
  }

  hf_solver_opts so;
  hf_default_opts(&so);
  so.precision = opt.precision;
  so.criterion = opt.criterion;
  so.tol = opt.tol > 0 ? opt.tol : (opt.criterion == HF_STOP_RECURSIVE ? 1e-32 : 1e-10);
  so.use_graph = opt.use_graph;
  hf_ctx* ctx = nullptr;
  int rc = hf_create(&deck.prob, &so, &ctx);
  if (rc != HF_OK) return fail_lib(rc, "hf_create");
  if (deck.tables.ntables() > 0) {
    const hfhost::PropertyTables& t = deck.tables;
    if ((rc = hf_set_property_tables(ctx, t.ntables(), t.offsets.data(), t.rows.data(),
                                     t.cell_table.data())) != HF_OK) {
      fail_lib(rc, "hf_set_property_tables");
      hf_destroy(ctx);
      return 1;
    }
  }
  std::printf(" Setup complete, running simulation\n");

  // initial_evolve
  std::vector<double> tp(n), tpp(n);
  try {
    if (P.full_restart) {
      tp = hfhost::parse_temp_file(hfhost::read_text_file(opt.restart + "/TempDis.dat", " Error: File not found: TempDis.dat"), n);
      tpp = hfhost::parse_temp_file(hfhost::read_text_file(opt.restart + "/TempDisTPD.dat", " Error: File not found: TempDisTPD.dat"), n);
    } else if (P.input_temp_dis) {
      tp = hfhost::parse_temp_file(hfhost::read_text_file(opt.restart + "/TempDis.dat", " Error: File not found: TempDis.dat"), n);
      tpp = tp;
    } else {
      std::fill(tp.begin(), tp.end(), P.t_system);
      std::fill(tpp.begin(), tpp.end(), P.t_system);
    }
  } catch (const hfhost::InputError& e) {
    std::printf(" %s\n", e.what());
    hf_destroy(ctx);
    return 1;
  }
  if ((rc = hf_set_state(ctx, tp.data(), tpp.data())) != HF_OK) {
    fail_lib(rc, "hf_set_state");
    hf_destroy(ctx);
    return 1;
  }

  mkdir(opt.outputs.c_str(), 0755);
  // sub-box of the log (1-based inclusive bounds of param.in; an empty box logs the time only)
  const int64_t lo[3] = {P.start_ix - 1, P.start_iy - 1, P.start_iz - 1};
  const int64_t hi[3] = {P.end_ix - 1, P.end_iy - 1, P.end_iz - 1};
  const bool box = hi[0] >= lo[0] && hi[1] >= lo[1] && hi[2] >= lo[2];
  const int64_t nbox = box ? (hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1) : 0;
  FILE* log = nullptr;
  auto final_print = [&]() -> int {
    int r = hf_get_state(ctx, tp.data(), tpp.data());
    if (r != HF_OK) return r;
    if (!write_file(opt.outputs + "/TempDis.dat", hfhost::format_temp_file(tp.data(), n)) ||
        !write_file(opt.outputs + "/TempDisTPD.dat", hfhost::format_temp_file(tpp.data(), n))) {
      std::fprintf(stderr, "cannot write %s/TempDis.dat\n", opt.outputs.c_str());
      return HF_EARG;
    }
    return HF_OK;
  };
  // data_write logs after step 1 and, with _WriteToTxt, every write_every steps (not in test
  // runs); step 1 gets two records when both rules apply (hfhost::records_after)
  auto logs_after = [&](int64_t it) { return hfhost::records_after(P, it) > 0; };
  // Log records in flight: the sub-box is gathered on the device after the step and copied to a
  // page-locked buffer on the library's second stream while the next steps run; records are
  // written in order once their copy is done (at most kInFlight at a time).
  constexpr int kInFlight = 3;
  struct Pending {
    int64_t itime = 0, ticket = -1;
    int slot = 0, copies = 1;   // the same record written `copies` times in a row
  };
  std::vector<std::vector<double>> ring(kInFlight + 1, std::vector<double>(nbox > 0 ? nbox : 1));
  for (auto& b : ring) hf_host_register(b.data(), b.size() * sizeof(double));   // best effort
  std::vector<Pending> pending;
  int next_slot = 0;
  auto drain = [&](size_t keep) -> int {
    while (pending.size() > keep) {
      const Pending p = pending.front();
      pending.erase(pending.begin());
      if (box) {
        const int r = hf_subbox_wait(ctx, p.ticket);
        if (r != HF_OK) return r;
      }
      const std::string rec = hfhost::format_record((double)(p.itime - 1) * P.time_step,
                                                    ring[p.slot].data(), nbox);
      for (int k = 0; k < p.copies; ++k) std::fwrite(rec.data(), 1, rec.size(), log);
    }
    return HF_OK;
  };
  auto cleanup = [&]() {
    for (auto& b : ring) hf_host_unregister(b.data());
    if (log) std::fclose(log);
    log = nullptr;
  };
  // a library error after set-up: the reference's message, then the buffers and the context go
  auto fail_run = [&](int r, const char* where) {
    fail_lib(r, where);
    cleanup();
    hf_destroy(ctx);
    return 1;
  };

  // The steps between two host actions (a log record, a per-step print at IVERB >= 3, the end)
  // run as one hf_run call: the whole loop as one CUDA graph launch.
  int64_t itime = 1;
  while (itime <= P.ntime) {
    int64_t last = itime;
    while (last < P.ntime && !logs_after(last) && P.iverb < 3) ++last;
    hf_stats st;
    rc = hf_run(ctx, itime, last - itime + 1, &st);
    if (rc != HF_OK) return fail_run(rc, "simulate");
    if (logs_after(last)) {
      if (last == 1) {
        log = std::fopen(hfhost::next_log_name(opt.outputs, P.run_name).c_str(), "w");
        if (!log) {
          std::fprintf(stderr, "cannot open the log in %s\n", opt.outputs.c_str());
          cleanup();
          hf_destroy(ctx);
          return 1;
        }
      }
      Pending p;
      p.itime = last;
      p.slot = next_slot;
      p.copies = hfhost::records_after(P, last);
      next_slot = (next_slot + 1) % (kInFlight + 1);
      // the _WriteToTxt record's message (mod_output.f90:110)
      if (P.write_to_txt && P.write_every > 0 && last % P.write_every == 0)
        std::printf(" Writing Temperature difference to file\n");
      if (box && (rc = hf_subbox_async(ctx, 0, lo, hi, 1, ring[p.slot].data(), &p.ticket)) != HF_OK)
        return fail_run(rc, "data_write");
      pending.push_back(p);
      if ((rc = drain(kInFlight - 1)) != HF_OK) return fail_run(rc, "data_write");
    }
    if (P.iverb >= 3 && (rc = final_print()) != HF_OK) return fail_run(rc, "final_print");
    if (last == P.ntime) {
      if ((rc = drain(0)) != HF_OK) return fail_run(rc, "data_write");
      if (log) std::fclose(log);
      log = nullptr;
      if ((rc = final_print()) != HF_OK) return fail_run(rc, "final_print");
    }
    itime = last + 1;
  }
  cleanup();
  hf_destroy(ctx);
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::printf(" time=%12.6f\n", secs);
  std::printf(" all done\n");
  return 0;
}
