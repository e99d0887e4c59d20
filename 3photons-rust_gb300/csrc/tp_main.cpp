// tp_main.cpp — `tp_run`, the command-line program of this library. It does
// what main() of 3photons-rust does (src/main.rs:75-145): read `valeurs`,
// run every batch (here on the GPU), merge them in batch order, finalise,
// print the reference's stdout and write res.data, res.times and pil.mc.
//
// usage: tp_run [-c valeurs] [-d output dir] [-n num_events] [--device D]
//               [--rng ranf|xoshiro] [--seed S] [--jump-per-batch]
//               [--no-photon-sorting] [--faster-evgen] [--fp32-mixed]
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/tp_gpu.h"

int main(int argc, char** argv) {
  std::string cfg_path = "valeurs", dir = ".";
  int kind = TP_RNG_RANF, flags = 0, device = 0, precision = TP_PREC_FP64;
  long long n_override = -1;
  bool seed_given = false;
  unsigned long long seed = 0;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    auto next = [&]() -> const char* {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "missing value after %s\n", a.c_str());
        std::exit(2);
      }
      return argv[++i];
    };
    if (a == "-c") cfg_path = next();
    else if (a == "-d") dir = next();
    else if (a == "-n") n_override = std::atoll(next());
    else if (a == "--device") device = std::atoi(next());
    else if (a == "--rng") kind = std::strcmp(next(), "ranf") == 0 ? TP_RNG_RANF : TP_RNG_XOSHIRO256P;
    else if (a == "--seed") { seed = std::strtoull(next(), nullptr, 10); seed_given = true; }
    else if (a == "--jump-per-batch") flags |= TP_MODE_JUMP_PER_BATCH;
    else if (a == "--no-photon-sorting") flags |= TP_MODE_NO_PHOTON_SORTING;
    else if (a == "--faster-evgen") flags |= TP_MODE_FASTER_EVGEN;
    else if (a == "--fp32-mixed") precision = TP_PREC_FP32_MIXED;
    else {
      std::fprintf(stderr, "unknown argument %s\n", a.c_str());
      return 2;
    }
  }
  if (!seed_given) seed = kind == TP_RNG_RANF ? TP_RANF_DEFAULT_SEED : TP_XOSHIRO_DEFAULT_SEED;
  tp_config cfg;
  std::vector<char> echo(4096);
  int st = tp_config_load(cfg_path.c_str(), &cfg, echo.data(), echo.size());
  std::fputs(echo.data(), stdout);
  if (st) {
    std::fprintf(stderr, "Error: failed to load the configuration (%d)\n", st);
    return 1;
  }
  if (n_override > 0) cfg.num_events = (uint64_t)n_override;
  const auto t0 = std::chrono::steady_clock::now();
  tp_ctx* ctx = tp_create(device, &st);
  if (!ctx) {
    std::fprintf(stderr, "Error: %s\n", tp_last_error(nullptr));
    return 1;
  }
  const uint64_t nb = (cfg.num_events + TP_BATCH_SIZE - 1) / TP_BATCH_SIZE;
  std::vector<uint64_t> sel(nb);
  std::vector<double> spm2(5 * nb), vars(5 * nb), sigma(nb), variance(nb);
  tp_batch_soa soa{sel.data(), spm2.data(), vars.data(), sigma.data(), variance.data()};
  st = tp_run_batches(ctx, &cfg, kind | flags, seed, 0, nb, precision, &soa);
  if (st) {
    std::fprintf(stderr, "Error: %s\n", tp_last_error(ctx));
    tp_destroy(ctx);
    return 1;
  }
  tp_destroy(ctx);
  tp_final_results res;
  st = tp_merge_finalize(&cfg, &soa, nb, &res);
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (st) return 1;
  std::vector<char> buf(1 << 16);
  tp_format_report(&cfg, &res, buf.data(), buf.size());
  std::fputs(buf.data(), stdout);
  if (tp_write_res_times(&cfg, secs, nullptr, (dir + "/res.times").c_str()) ||
      tp_write_res_data(&cfg, &res, (dir + "/res.data").c_str()) ||
      tp_append_pil_mc(&cfg, &res, nullptr, (dir + "/pil.mc").c_str())) {
    std::fprintf(stderr, "Error: failed to output the results\n");
    return 1;
  }
  return 0;
}
