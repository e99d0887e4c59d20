// tp_oracle_main.cpp — command-line driver of the CPU restatement, mirroring
// main() of 3photons-rust (src/main.rs:75-145): reads `valeurs`, runs every
// batch, merges them in order, writes res.data and prints the stdout of the
// reference. Test infrastructure only.
//
// usage: tp_oracle [-c valeurs] [-o res.data] [-n num_events]
//                  [--rng ranf|xoshiro] [--seed S] [--jump-per-batch]
//                  [--no-photon-sorting] [--faster-evgen] [--threads T]
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "tp_oracle.h"

int main(int argc, char** argv) {
  std::string cfg_path = "valeurs", out_path = "res.data";
  int kind = TP_RNG_RANF, flags = 0, threads = 1;
  long long n_override = -1;
  bool seed_given = false;
  unsigned long long seed = 0;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&]() -> const char* {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "missing value after %s\n", a.c_str());
        std::exit(2);
      }
      return argv[++i];
    };
    if (a == "-c") cfg_path = next();
    else if (a == "-o") out_path = next();
    else if (a == "-n") n_override = std::atoll(next());
    else if (a == "--rng") kind = std::strcmp(next(), "ranf") == 0 ? TP_RNG_RANF : TP_RNG_XOSHIRO256P;
    else if (a == "--seed") { seed = std::strtoull(next(), nullptr, 10); seed_given = true; }
    else if (a == "--jump-per-batch") flags |= TP_MODE_JUMP_PER_BATCH;
    else if (a == "--no-photon-sorting") flags |= TP_MODE_NO_PHOTON_SORTING;
    else if (a == "--faster-evgen") flags |= TPO_MODE_FASTER_EVGEN;
    else if (a == "--threads") threads = std::atoi(next());
    else {
      std::fprintf(stderr, "unknown argument %s\n", a.c_str());
      return 2;
    }
  }
  if (!seed_given) seed = kind == TP_RNG_RANF ? TP_RANF_DEFAULT_SEED : TP_XOSHIRO_DEFAULT_SEED;
  tp_config cfg;
  std::vector<char> echo(4096);
  int st = tpo_config_load(cfg_path.c_str(), &cfg, echo.data(), echo.size());
  std::fputs(echo.data(), stdout);
  if (st) {
    std::fprintf(stderr, "failed to load the configuration (%d)\n", st);
    return 1;
  }
  if (n_override > 0) cfg.num_events = (uint64_t)n_override;
  auto t0 = std::chrono::steady_clock::now();
  const uint64_t nb = (cfg.num_events + TP_BATCH_SIZE - 1) / TP_BATCH_SIZE;
  std::vector<uint64_t> sel(nb);
  std::vector<double> spm2(5 * nb), vars(5 * nb), sigma(nb), variance(nb);
  tp_batch_soa soa{sel.data(), spm2.data(), vars.data(), sigma.data(), variance.data()};
  st = tpo_run_batches(&cfg, kind | flags, seed, 0, nb, &soa, threads);
  if (st) return 1;
  tp_final_results res;
  tpo_merge_finalize(&cfg, &soa, nb, &res);
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::vector<char> buf(1 << 16);
  tpo_format_report(&cfg, &res, buf.data(), buf.size());
  std::fputs(buf.data(), stdout);
  tpo_format_res_data(&cfg, &res, buf.data(), buf.size());
  FILE* f = std::fopen(out_path.c_str(), "w");
  if (!f) return 1;
  std::fputs(buf.data(), f);
  std::fclose(f);
  std::fprintf(stderr, "elapsed %.3f s, %.4g events/s\n", secs, cfg.num_events / secs);
  return 0;
}
