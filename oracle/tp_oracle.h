// tp_oracle.h — C ABI of the CPU restatement of 3photons-rust (test
// infrastructure only: the checker and CPU baseline, never the product).
#ifndef TP_ORACLE_H
#define TP_ORACLE_H

#include "../include/tp_gpu.h"

// Oracle-only mode flag: `--features faster-evgen` (src/evgen.rs:143-173).
#define TPO_MODE_FASTER_EVGEN 0x400

#ifdef __cplusplus
extern "C" {
#endif

int tpo_config_load(const char* path, tp_config* out, char* echo, size_t echo_len);
double tpo_event_weight(double e_total);
void tpo_couplings(const tp_config* cfg, double out[3]);
void tpo_sigma_contribs(const tp_config* cfg, double out[5]);
int tpo_draws(int rng_kind, uint64_t seed, uint64_t jumps, uint64_t skip, uint64_t n, double* out);
void tpo_xoshiro_state(uint64_t seed, uint64_t jumps, uint64_t state[4]);
void tpo_xoshiro_jump128(uint64_t state[4]);
void tpo_ranf_state(int32_t seed, uint64_t resets, int32_t out[56]);
int tpo_dump_events(const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_event, uint64_t n,
                    tp_event_dump* out);
void tpo_m2_sums_of(const tp_config* cfg, const double* p_out, double out[5]);
int tpo_run_batches(const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_batch, uint64_t n_batches,
                    tp_batch_soa* out, int threads);
// tpo_run_batches for a stream that starts from `seed` jumped `jumps` times
// (RandomGenerator::jump): the stream of parameter point `jumps` of a scan.
int tpo_run_batches_jumped(const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t jumps, uint64_t first_batch,
                           uint64_t n_batches, tp_batch_soa* out, int threads);
int tpo_binned(const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_batch, uint64_t n_batches, int nx,
               int ny, double xlo, double xhi, double ylo, double yhi, double* out);
int tpo_merge_finalize(const tp_config* cfg, const tp_batch_soa* b, uint64_t n, tp_final_results* res);
int tpo_format_res_data(const tp_config* cfg, const tp_final_results* r, char* buf, size_t len);
int tpo_format_report(const tp_config* cfg, const tp_final_results* r, char* buf, size_t len);

#ifdef __cplusplus
}
#endif

#endif
