// tp_host.cpp — the host side the reference keeps around its event loop:
// the `valeurs` parser and echo (src/config.rs:57-155), the per-run
// constants (src/evgen.rs:40-77, src/coupling.rs:23-33, src/resacc.rs:59-117),
// the ordered merge and finalisation (src/resacc.rs:133-223) and the
// res.data / report writers (src/output.rs:30-269, src/resfin.rs:66-194).
//
// Floating-point expressions follow the reference's operation order; powi
// is square-and-multiply (LLVM's lowering); powers of constants are folded
// with pow() as rustc's constant folding does.
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "tp_internal.h"

namespace tp {
namespace {

double powi(double a, int b) {
  const bool recip = b < 0;
  if (recip) b = -b;
  double r = 1.0;
  for (;;) {
    if (b & 1) r *= a;
    b /= 2;
    if (b == 0) break;
    a *= a;
  }
  return recip ? 1.0 / r : r;
}

constexpr double kSqrt2 = 1.41421356237309504880168872420969808;
constexpr double kFracPi2 = 1.57079632679489661923132169163975144;

// Constants of ResultsAccumulator::new (src/resacc.rs:59-117)
struct RunConsts {
  double fact_com, norm_weight, propagator, delta;
  double sc[5];
};

RunConsts run_consts(const tp_config& cfg) {
  RunConsts r{};
  const double fact_com = (1.0 / 6.0) * cfg.gev2_to_picobarn;
  const double relat_width = cfg.g_z0 / cfg.m_z0;
  const double p_aa = 2.0;
  const double p_ab = 1.0 - 4.0 * cfg.sin2_weinberg;
  const double p_bb = p_ab + 8.0 * powi(cfg.sin2_weinberg, 2);
  const double c_aa = fact_com * p_aa;
  const double c_ab = fact_com * p_ab / powi(cfg.m_z0, 2);
  const double c_bb = fact_com * p_bb / powi(cfg.m_z0, 4);
  const double dzeta = powi(cfg.e_total / cfg.m_z0, 2);
  const double delta = (dzeta - 1.0) / relat_width;
  const double propagator = 1.0 / (1.0 + powi(delta, 2));
  const double n_ev = (double)cfg.num_events;
  const double norm = std::pow(2.0 * kPi, -5.0) / n_ev;  // (2 PI)^(4 - 3*3)
  const double norm_weight = event_weight(cfg.e_total) * norm;
  const double com = norm_weight / 4.0;
  const double aa = com * c_aa;
  const double bb = com * c_bb * propagator / powi(relat_width, 2);
  const double ab = com * c_ab * 2.0 * cfg.beta_plus * propagator / relat_width;
  r.sc[0] = aa;
  r.sc[1] = bb * powi(cfg.beta_plus, 2);
  r.sc[2] = bb * powi(cfg.beta_minus, 2);
  r.sc[3] = ab * delta;
  r.sc[4] = -ab;
  r.fact_com = fact_com;
  r.norm_weight = norm_weight;
  r.propagator = propagator;
  r.delta = delta;
  return r;
}

// ---------------------------------------------------------------------------
// Rust float formatting. The goldens print zero without its sign.
// ---------------------------------------------------------------------------
std::string fmt_fixed(double x, int prec) {
  if (std::isnan(x)) return "NaN";
  if (std::isinf(x)) return x > 0 ? "inf" : "-inf";
  if (x == 0.0) x = 0.0;
  char buf[512];
  std::snprintf(buf, sizeof buf, "%.*f", prec, x);
  return buf;
}

std::string fmt_exp(double x, int prec) {  // {:.prec$e}: "1.2345e-4"
  if (std::isnan(x)) return "NaN";
  if (std::isinf(x)) return x > 0 ? "inf" : "-inf";
  if (x == 0.0) x = 0.0;
  char buf[512];
  std::snprintf(buf, sizeof buf, "%.*e", prec, x);
  const char* e = std::strchr(buf, 'e');
  return std::string(buf, (size_t)(e - buf)) + "e" + std::to_string(std::atoi(e + 1));
}

std::string fmt_display(double x) {  // {}: shortest round-trip, positional
  if (std::isnan(x)) return "NaN";
  if (std::isinf(x)) return x > 0 ? "inf" : "-inf";
  if (x == 0.0) return "0";
  char buf[512];
  const auto r = std::to_chars(buf, buf + sizeof buf, x, std::chars_format::fixed);
  return std::string(buf, r.ptr);
}

std::string lpad(const std::string& s, size_t w) {
  return s.size() >= w ? s : std::string(w - s.size(), ' ') + s;
}

// write_engineering (src/output.rs:230-269), SIG_DIGITS = f64::DIGITS - 1
std::string fmt_engineering(double x) {
  const int sig_digits = 14;
  long precision = sig_digits - 1;
  if (x == 0.0) return "0";
  const double log_x = std::log10(std::fabs(x));
  if (log_x >= -3.0 && log_x <= (double)sig_digits) {
    precision -= (long)std::trunc(log_x);
    if (log_x < 0.0) precision += 1;
    std::string s = fmt_fixed(x, (int)precision);
    if (s.find('.') != std::string::npos) {
      s.erase(s.find_last_not_of('0') + 1);
      if (!s.empty() && s.back() == '.') s.pop_back();
    }
    return s;
  }
  return fmt_exp(x, (int)precision);
}

// writeln_3p for (key, value) pairs (src/output.rs:179-220)
void kv(std::string& s, const char* key, const std::string& val) {
  std::string k(key);
  if (k.size() < 31) k.append(31 - k.size(), ' ');
  s += " " + k + ": " + val + "\n";
}

int copy_out(const std::string& s, char* buf, size_t len) {
  if (buf && len) {
    const size_t n = s.size() < len - 1 ? s.size() : len - 1;
    std::memcpy(buf, s.data(), n);
    buf[n] = 0;
  }
  return (int)s.size();
}

std::string res_data_text(const tp_config& cfg, const tp_final_results& r) {
  std::string s;
  kv(s, "Nombre d'evenements", std::to_string(cfg.num_events));
  kv(s, "... apres coupure", std::to_string(r.selected_events));
  kv(s, "energie dans le CdM      (GeV)", fmt_engineering(cfg.e_total));
  kv(s, "coupure / cos(photon,faisceau)", fmt_engineering(cfg.beam_photons_cut));
  kv(s, "coupure / cos(photon,photon)", fmt_engineering(cfg.photon_photon_cut));
  kv(s, "coupure / sin(normale,faisceau)", fmt_engineering(cfg.beam_photon_plane_cut));
  kv(s, "coupure sur l'energie    (GeV)", fmt_engineering(cfg.e_min));
  kv(s, "1/(constante de structure fine)", fmt_engineering(1.0 / cfg.alpha));
  kv(s, "1/(structure fine au pic)", fmt_engineering(1.0 / cfg.alpha_z));
  kv(s, "facteur de conversion GeV-2/pb", fmt_engineering(cfg.gev2_to_picobarn));
  kv(s, "Masse du Z0              (GeV)", fmt_engineering(cfg.m_z0));
  kv(s, "Largeur du Z0            (GeV)", fmt_engineering(cfg.g_z0));
  kv(s, "Sinus^2 Theta Weinberg", fmt_engineering(cfg.sin2_weinberg));
  kv(s, "Taux de branchement Z--->e+e-", fmt_engineering(cfg.branching_ep_em));
  kv(s, "Beta plus", fmt_engineering(cfg.beta_plus));
  kv(s, "Beta moins", fmt_engineering(cfg.beta_minus));
  s += " ---------------------------------------------\n";
  kv(s, "Section Efficace          (pb)", fmt_engineering(r.sigma));
  kv(s, "Ecart-Type                (pb)", fmt_engineering(r.sigma * r.prec));
  kv(s, "Precision Relative", fmt_engineering(r.prec));
  s += " ---------------------------------------------\n";
  kv(s, "Beta minimum", fmt_engineering(r.beta_min));
  kv(s, "Stat. Significance  B+(pb-1/2)", fmt_engineering(r.ss_p));
  kv(s, "Incert. Stat. Sign. B+(pb-1/2)", fmt_engineering(r.ss_p * r.inc_ss_p));
  kv(s, "Stat. Significance  B-(pb-1/2)", fmt_engineering(r.ss_m));
  kv(s, "Incert. Stat. Sign. B-(pb-1/2)", fmt_engineering(r.ss_m * r.inc_ss_m));
  s += "\n";
  const int decs = 7;  // min(SIG_DIGITS - 1, 7)
  const size_t width = decs + 8;
  for (int sp = 0; sp < 2; ++sp) {
    for (int c = 0; c < 5; ++c) {
      s += lpad(std::to_string(sp + 1), 3) + lpad(std::to_string(c + 1), 3);
      s += lpad(fmt_exp(r.spm2[sp][c], decs), width);
      s += lpad(fmt_exp(std::fabs(r.spm2[sp][c]) * r.vars[sp][c], decs), width);
      s += lpad(fmt_exp(r.vars[sp][c], decs), width) + "\n";
    }
    s += "\n";
  }
  for (int c = 0; c < 5; ++c) {
    const double tmp1 = (0.0 + r.spm2[0][c]) + r.spm2[1][c];
    const double a = r.spm2[0][c] * r.vars[0][c];
    const double b = r.spm2[1][c] * r.vars[1][c];
    const double tmp2 = std::sqrt(0.0 + (a * a + b * b));
    s += "   " + lpad(std::to_string(c + 1), 3);
    s += lpad(fmt_exp(tmp1 / 4.0, decs), width);
    s += lpad(fmt_exp(tmp2 / 4.0, decs), width);
    s += lpad(fmt_exp(tmp2 / std::fabs(tmp1), decs), width) + "\n";
  }
  return s;
}

}  // namespace

double event_weight(double e_total) {
  // EventGenerator::new (src/evgen.rs:40-77), 3 outgoing photons
  double z_n = (3.0 - 1.0) * std::log(kFracPi2);
  z_n -= 2.0 * std::log(1.0);
  z_n = z_n - std::log(2.0);
  const double ln_weight = (2.0 * 3.0 - 4.0) * std::log(e_total) + z_n;
  return std::exp(ln_weight);
}

int check_config(const tp_config* cfg) {
  if (!cfg) return TP_ERR_INVALID;
  if (cfg->num_events == 0) return TP_ERR_INVALID;
  if (!(cfg->e_total > 0.0) || !std::isfinite(cfg->e_total)) return TP_ERR_INVALID;
  if (cfg->impr || cfg->plot) return TP_ERR_INVALID;
  // the event weight's range check (src/evgen.rs:61)
  const double lw = std::log(event_weight(cfg->e_total));
  if (!(lw >= -180.0 && lw <= 174.0)) return TP_ERR_INVALID;
  return TP_OK;
}

int make_ev_const(const tp_config& cfg, int flags, EvConst* out) {
  EvConst k{};
  k.e_total = cfg.e_total;
  k.half = cfg.e_total / 2.0;
  k.em_x = -cfg.e_total / 2.0;
  k.acut = cfg.beam_photons_cut;
  k.bcut = cfg.photon_photon_cut;
  k.emin = cfg.e_min;
  k.sincut = cfg.beam_photon_plane_cut;
  // Couplings::new (src/coupling.rs:23-33)
  const double e2 = (4.0 * kPi) * cfg.alpha;
  const double e2_z = (4.0 * kPi) * cfg.alpha_z;
  const double cos2w = 1.0 - cfg.sin2_weinberg;
  const double g_beta = -std::sqrt(e2_z / ((4.0 * cos2w) * cfg.sin2_weinberg)) / powi(cfg.m_z0, 4);
  k.g_a = -powi(std::sqrt(e2), 3);
  k.g_bp = g_beta;
  k.g_bm = g_beta;
  const RunConsts rc = run_consts(cfg);
  for (int c = 0; c < 5; ++c) k.sc[c] = rc.sc[c];
  // beams: p = (-+E/2, 0, 0, E/2), so xx = sqrt(E/2 + 0) and fx = p_x / xx
  k.xx_in = std::sqrt(k.half + 0.0);
  k.fx_em = k.em_x / k.xx_in;
  k.fx_ep = k.half / k.xx_in;
  k.s01 = k.fx_em * k.xx_in - k.fx_ep * k.xx_in;
  const double rac8 = 2.0 * kSqrt2;
  k.c1 = -rac8 * k.s01;
  k.c2 = -k.c1;
  k.sc_raw[0] = (k.g_a * k.c1) * (k.g_a * k.c1);
  k.sc_raw[1] = (k.g_bp * k.c1) * (k.g_bp * k.c1);
  k.sc_raw[2] = (k.g_bm * k.c1) * (k.g_bm * k.c1);
  k.sc_raw[3] = -2.0 * k.g_a * k.g_bp * k.c1 * k.c1;
  k.f_e_total = (float)k.e_total;
  k.f_half = (float)k.half;
  k.f_em_x = (float)k.em_x;
  k.f_acut = (float)k.acut;
  k.f_acut_half = (float)(k.acut * k.half);
  k.f_bcut = (float)k.bcut;
  k.f_emin = (float)k.emin;
  k.f_sincut = (float)k.sincut;
  k.f_xx_in = (float)k.xx_in;
  k.f_fx_em = (float)k.fx_em;
  k.f_fx_ep = (float)k.fx_ep;
  k.f_c1 = (float)k.c1;
  k.f_c2 = (float)k.c2;
  // the FP32 sums' scaling: momenta in units of lambda (a power of 2 at
  // least the beam energy); with gamma = xx_in lambda the five sums are
  // homogeneous of degrees gamma^-4 lambda^2, gamma^4 lambda^2 (twice) and
  // lambda^2 (twice) in the spinor normalisation
  int lexp = 0;
  std::frexp(k.half, &lexp);  // half = f 2^lexp, 0.5 <= f < 1
  const double lambda = std::ldexp(1.0, lexp);
  const double gamma = k.xx_in * lambda, g4 = gamma * gamma * gamma * gamma, l2 = lambda * lambda;
  const double hat[5] = {l2 / g4, g4 * l2, g4 * l2, l2, l2};
  k.f_inv_lambda = (float)(1.0 / lambda);
  for (int c = 0; c < 5; ++c) {
    k.hat_scale[c] = hat[c];
    k.sc_raw_hat[c] = k.sc_raw[c < 3 ? c : 3] * hat[c];
    k.f_sc_raw[c] = (float)k.sc_raw_hat[c];
    k.f_raw_to_hat[c] = (float)(1.0 / hat[c]);
    k.f_raw_to_hat_lo[c] = (float)(1.0 / hat[c] - (double)k.f_raw_to_hat[c]);
  }
  for (int c = 0; c < 5; ++c) k.f_sc[c] = (float)k.sc[c];
  for (int c = 0; c < 5; ++c) {
    k.K[c] = k.sc_raw[c < 3 ? c : 3] * k.sc[c];
    k.f_K[c] = (float)(k.K[c] * hat[c]);
  }
  k.flags = flags;
  *out = k;
  return TP_OK;
}

}  // namespace tp

using namespace tp;

extern "C" {

int tp_config_load(const char* path, tp_config* out, char* echo, size_t echo_len) {
  if (!path || !out) return TP_ERR_INVALID;
  std::ifstream f(path);
  if (!f) return TP_ERR_IO;
  std::vector<std::string> items;
  std::string line;
  while (items.size() < 18 && std::getline(f, line)) {
    std::istringstream ls(line);
    std::string tok;
    if (ls >> tok) items.push_back(tok);
  }
  if (items.size() < 18) return TP_ERR_INVALID;
  tp_config c{};
  {
    const std::string& t = items[0];
    const char* b = t.c_str() + (t[0] == '+' ? 1 : 0);
    const auto r = std::from_chars(b, t.c_str() + t.size(), c.num_events);
    if (r.ec != std::errc() || r.ptr != t.c_str() + t.size()) return TP_ERR_INVALID;
  }
  double* dst[14] = {&c.e_total, &c.beam_photons_cut, &c.photon_photon_cut, &c.e_min,
                     &c.beam_photon_plane_cut, &c.alpha, &c.alpha_z, &c.gev2_to_picobarn,
                     &c.m_z0, &c.g_z0, &c.sin2_weinberg, &c.branching_ep_em,
                     &c.beta_plus, &c.beta_minus};
  for (int i = 0; i < 14; ++i) {
    char* end = nullptr;
    *dst[i] = std::strtod(items[1 + i].c_str(), &end);
    if (!end || *end) return TP_ERR_INVALID;
  }
  {
    char* end = nullptr;
    const long nb = std::strtol(items[15].c_str(), &end, 10);
    if (!end || *end) return TP_ERR_INVALID;
    c.num_bins = (int32_t)nb;
  }
  for (int i = 16; i < 18; ++i) {
    std::string t = items[i];
    for (auto& ch : t) ch = (char)std::tolower((unsigned char)ch);
    int32_t v;
    if (t == ".true." || t == "true") v = 1;
    else if (t == ".false." || t == "false") v = 0;
    else return TP_ERR_INVALID;
    (i == 16 ? c.impr : c.plot) = v;
  }
  if (echo && echo_len) {
    std::string s;
    s += "ITOT           : " + std::to_string(c.num_events) + "\n";
    s += "ETOT           : " + fmt_display(c.e_total) + "\n";
    s += "oCutpar.ACUT   : " + fmt_display(c.beam_photons_cut) + "\n";
    s += "oCutpar.BCUT   : " + fmt_display(c.photon_photon_cut) + "\n";
    s += "oCutpar.EMIN   : " + fmt_display(c.e_min) + "\n";
    s += "oCutpar.SINCUT : " + fmt_display(c.beam_photon_plane_cut) + "\n";
    s += "ALPHA          : " + fmt_display(c.alpha) + "\n";
    s += "ALPHAZ         : " + fmt_display(c.alpha_z) + "\n";
    s += "CONVERS        : " + fmt_display(c.gev2_to_picobarn) + "\n";
    s += "oParam.MZ0     : " + fmt_display(c.m_z0) + "\n";
    s += "oParam.GZ0     : " + fmt_display(c.g_z0) + "\n";
    s += "SIN2W          : " + fmt_display(c.sin2_weinberg) + "\n";
    s += "BREPEM         : " + fmt_display(c.branching_ep_em) + "\n";
    s += "BETAPLUS       : " + fmt_display(c.beta_plus) + "\n";
    s += "BETAMOINS      : " + fmt_display(c.beta_minus) + "\n";
    s += "NBIN           : " + std::to_string(c.num_bins) + "\n";
    s += std::string("oParam.IMPR    : ") + (c.impr ? "true" : "false") + "\n";
    s += std::string("PLOT           : ") + (c.plot ? "true" : "false") + "\n";
    copy_out(s, echo, echo_len);
  }
  *out = c;
  // the reference echoes first, then applies its checks (src/config.rs:110-124)
  if (c.num_events == 0 || c.plot || c.impr) return TP_ERR_INVALID;
  return TP_OK;
}

int tp_event_weight(double e_total, double* weight) {
  if (!weight || !(e_total > 0.0)) return TP_ERR_INVALID;
  *weight = event_weight(e_total);
  return TP_OK;
}

int tp_merge_finalize(const tp_config* cfg, const tp_batch_soa* b, uint64_t n, tp_final_results* res) {
  if (check_config(cfg) || !b || !res || n == 0) return TP_ERR_INVALID;
  if (!b->selected || !b->spm2 || !b->vars || !b->sigma || !b->variance) return TP_ERR_INVALID;
  const RunConsts rc = run_consts(*cfg);
  // ResultsAccumulator::merge, batch order (src/resacc.rs:133-139)
  uint64_t selected = 0;
  double spm2[5] = {0, 0, 0, 0, 0}, vars[5] = {0, 0, 0, 0, 0}, sigma = 0.0, variance = 0.0;
  for (uint64_t i = 0; i < n; ++i) {
    selected += b->selected[i];
    for (int c = 0; c < 5; ++c) spm2[c] += b->spm2[c * n + i];
    for (int c = 0; c < 5; ++c) vars[c] += b->vars[c * n + i];
    sigma += b->sigma[i];
    variance += b->variance[i];
  }
  // ResultsAccumulator::finalize (src/resacc.rs:142-223)
  const double n_ev = (double)cfg->num_events;
  for (int c = 0; c < 5; ++c) {
    double v = (vars[c] - powi(spm2[c], 2) / n_ev) / (n_ev - 1.0);
    vars[c] = std::sqrt(v / n_ev) / std::fabs(spm2[c] / n_ev);
  }
  double m[2][5];
  for (int s = 0; s < 2; ++s)
    for (int c = 0; c < 5; ++c) {
      m[s][c] = spm2[c];
      res->vars[s][c] = vars[c];
    }
  const double polar_p = -2.0 * cfg->sin2_weinberg;
  const double polars[2] = {1.0 + polar_p, polar_p};
  for (int c = 1; c < 5; ++c)
    for (int s = 0; s < 2; ++s) m[s][c] *= polars[s];
  for (int c = 1; c < 3; ++c)
    for (int s = 0; s < 2; ++s) m[s][c] *= polars[s];
  const double flux = 1.0 / (2.0 * powi(cfg->e_total, 2));
  const double f = rc.fact_com * flux * rc.norm_weight;
  for (int s = 0; s < 2; ++s)
    for (int c = 0; c < 5; ++c) m[s][c] *= f;
  const double gm_z0 = cfg->g_z0 * cfg->m_z0;
  const double pg = rc.propagator / gm_z0;
  for (int c = 1; c < 5; ++c)
    for (int s = 0; s < 2; ++s) m[s][c] *= pg;
  for (int c = 1; c < 3; ++c)
    for (int s = 0; s < 2; ++s) m[s][c] /= gm_z0;
  for (int s = 0; s < 2; ++s) m[s][3] *= rc.delta;
  auto colsum = [&](int c) { return (0.0 + m[0][c]) + m[1][c]; };
  auto inc_num = [&](int c) {
    const double a = m[0][c] * res->vars[0][c];
    const double bb = m[1][c] * res->vars[1][c];
    return std::sqrt(0.0 + (a * a + bb * bb));
  };
  res->beta_min = std::sqrt(colsum(0) / colsum(1));
  const double ss_denom = colsum(0);
  const double ss_norm = 1.0 / (2.0 * std::sqrt(ss_denom));
  res->ss_p = colsum(1) * ss_norm;
  res->ss_m = colsum(2) * ss_norm;
  const double inc_common = inc_num(0) / (2.0 * std::fabs(ss_denom));
  res->inc_ss_p = inc_num(1) / std::fabs(colsum(1)) + inc_common;
  res->inc_ss_m = inc_num(2) / std::fabs(colsum(2)) + inc_common;
  const double var = (variance - powi(sigma, 2) / n_ev) / (n_ev - 1.0);
  res->variance = var;
  res->prec = std::sqrt(var / n_ev) / std::fabs(sigma / n_ev);
  res->sigma = sigma * flux;
  res->selected_events = selected;
  for (int s = 0; s < 2; ++s)
    for (int c = 0; c < 5; ++c) res->spm2[s][c] = m[s][c];
  return TP_OK;
}

int tp_format_res_data(const tp_config* cfg, const tp_final_results* res, char* buf, size_t len) {
  if (!cfg || !res) return TP_ERR_INVALID;
  return copy_out(res_data_text(*cfg, *res), buf, len);
}

int tp_write_res_data(const tp_config* cfg, const tp_final_results* res, const char* path) {
  if (!cfg || !res || !path) return TP_ERR_INVALID;
  const std::string s = res_data_text(*cfg, *res);
  FILE* f = std::fopen(path, "w");
  if (!f) return TP_ERR_IO;
  const size_t w = std::fwrite(s.data(), 1, s.size(), f);
  const int closed = std::fclose(f);
  return (w == s.size() && closed == 0) ? TP_OK : TP_ERR_IO;
}

namespace {
std::string utc_stamp(const char* given) {
  if (given) return given;
  static const char* mon[12] = {"Jan", "Feb", "Mar", "Apr", "May", "Jun",
                                "Jul", "Aug", "Sep", "Oct", "Nov", "Dec"};
  const time_t now = time(nullptr);
  struct tm t;
  gmtime_r(&now, &t);
  char buf[64];
  std::snprintf(buf, sizeof buf, "%02d-%s-%02d %02d:%02d:%02d", t.tm_mday, mon[t.tm_mon], t.tm_year % 100,
                t.tm_hour, t.tm_min, t.tm_sec);
  return buf;
}
}  // namespace

int tp_write_res_times(const tp_config* cfg, double elapsed, const char* timestamp, const char* path) {
  if (!cfg || !path) return TP_ERR_INVALID;
  std::string s = " " + utc_stamp(timestamp) + "\n";
  s += " ---------------------------------------------\n";
  kv(s, "Temps ecoule", "???");
  kv(s, "Temps ecoule utilisateur", fmt_engineering(elapsed));
  kv(s, "Temps ecoule systeme", "???");
  kv(s, "Temps ecoule par evenement", fmt_engineering(elapsed / (double)cfg->num_events));
  FILE* f = std::fopen(path, "w");
  if (!f) return TP_ERR_IO;
  const size_t w = std::fwrite(s.data(), 1, s.size(), f);
  return (std::fclose(f) == 0 && w == s.size()) ? TP_OK : TP_ERR_IO;
}

int tp_append_pil_mc(const tp_config* cfg, const tp_final_results* r, const char* timestamp, const char* path) {
  if (!cfg || !r || !path) return TP_ERR_INVALID;
  auto colsum = [&](int c) { return (0.0 + r->spm2[0][c]) + r->spm2[1][c]; };
  const double res1 = colsum(0);
  const double res2 = colsum(1) * powi(cfg->beta_plus, 2);
  const double res3 = colsum(2) * powi(cfg->beta_minus, 2);
  const double res4 = colsum(3) * cfg->beta_plus;
  std::string s = utc_stamp(timestamp) + "\n";
  s += fmt_display(cfg->e_total) + " " + fmt_display(res1 / 4.0) + " " + fmt_display(res2 / 4.0) + " " +
       fmt_display(res3 / 4.0) + " " + fmt_display(res4 / 4.0) + " " +
       fmt_display((res1 + res2 + res3 + res4) / 4.0) + " " + fmt_display(r->sigma) + "\n";
  FILE* f = std::fopen(path, "a");
  if (!f) return TP_ERR_IO;
  const size_t w = std::fwrite(s.data(), 1, s.size(), f);
  return (std::fclose(f) == 0 && w == s.size()) ? TP_OK : TP_ERR_IO;
}

int tp_format_report(const tp_config* cfg, const tp_final_results* r, char* buf, size_t len) {
  if (!cfg || !r) return TP_ERR_INVALID;
  std::string s = "IBegin\n";
  auto line = [&](const std::string& l) { s += l + "\n"; };
  const auto& m = r->spm2;
  // FinalResults::eric (src/resfin.rs:66-97)
  const double mu_th = cfg->branching_ep_em * cfg->gev2_to_picobarn /
                       ((8.0 * 9.0 * 5.0 * std::pow(kPi, 2.0)) * cfg->m_z0 * cfg->g_z0);
  double sigma0[2], alpha0[2], beta0[2], lambda0[2], mu0[2];
  for (int sp = 0; sp < 2; ++sp) {
    sigma0[sp] = m[sp][0] / 2.0;
    alpha0[sp] = m[sp][4] / 2.0;
    beta0[sp] = -m[sp][3] / 2.0;
    lambda0[sp] = (m[sp][2] - m[sp][1]) / 2.0;
    mu0[sp] = (m[sp][2] + m[sp][1]) / 2.0;
  }
  const double mu_num = ((((0.0 + m[0][1]) + m[1][1]) + m[0][2]) + m[1][2]) / 4.0;
  line("");
  line("       :        -          +");
  line("sigma0  : " + fmt_fixed(sigma0[0], 6) + " | " + fmt_fixed(sigma0[1], 6));
  line("alpha0  : " + fmt_exp(alpha0[0], 5) + " | " + fmt_exp(alpha0[1], 4));
  line("beta0   : " + fmt_display(beta0[0]) + " | " + fmt_display(beta0[1]));
  line("lambda0 : " + fmt_fixed(lambda0[0], 4) + " | " + fmt_fixed(lambda0[1], 4));
  line("mu0     : " + fmt_fixed(mu0[0], 4) + " | " + fmt_fixed(mu0[1], 5));
  line("mu/lamb : " + fmt_fixed(mu0[0] / lambda0[0], 5) + " | " + fmt_fixed(mu0[1] / lambda0[1], 5));
  line("mu (num): " + fmt_fixed(mu_num, 4));
  line("rapport : " + fmt_fixed(mu_num / mu_th, 6));
  line("mu (th) : " + fmt_fixed(mu_th, 4));
  // FinalResults::fawzi (src/resfin.rs:101-194)
  const double mre = cfg->m_z0 / cfg->e_total;
  const double gre = cfg->g_z0 * cfg->m_z0 / powi(cfg->e_total, 2);
  const double x = 1.0 - powi(mre, 2);
  const double sd = powi(x, 2) + powi(gre, 2);
  const double sdz_re = x / sd, sdz_im = -gre / sd;
  const double del = (1.0 - cfg->photon_photon_cut) / 2.0;
  const double eps = 2.0 * cfg->e_min / cfg->e_total;
  const double bra = cfg->m_z0 / (3.0 * 6.0 * std::pow(kPi, 3.0) * 16.0 * 120.0);
  const double sig = 12.0 * kPi / powi(cfg->m_z0, 2) * cfg->branching_ep_em * cfg->g_z0 * bra /
                     powi(cfg->e_total, 2) * powi(cfg->e_total / cfg->m_z0, 8) *
                     (sdz_re * sdz_re + sdz_im * sdz_im) * cfg->gev2_to_picobarn;
  const double eps_4 = powi(eps, 4);
  const double del_2 = powi(del, 2);
  const double del_3 = powi(del, 3);
  const double f1 = 1.0 - 15.0 * eps_4 - 9.0 / 7.0 * (1.0 - 70.0 * eps_4) * del_2 +
                    6.0 / 7.0 * (1.0 + 70.0 * eps_4) * del_3;
  const double g1 = 1.0 - 30.0 * eps_4 - 9.0 / 7.0 * (1.0 - 70.0 * eps_4) * del - 90.0 * eps_4 * del_2 -
                    1.0 / 7.0 * (1.0 - 420.0 * eps_4) * del_3;
  const double g2 = 1.0 - 25.0 * eps_4 - 6.0 / 7.0 * (1.0 - 70.0 * eps_4) * del -
                    3.0 / 7.0 * (1.0 + 210.0 * eps_4) * del_2 - 8.0 / 21.0 * (1.0 - 52.5 * eps_4) * del_3;
  const double g3 = 1.0 - 195.0 / 11.0 * eps_4 - 18.0 / 77.0 * (1.0 - 7.0 * eps_4) * del -
                    9.0 / 11.0 * (9.0 / 7.0 - 70.0 * eps_4) * del_2 -
                    8.0 / 11.0 * (1.0 - 105.0 / 11.0 * eps_4) * del_3;
  const double sc3 = powi(cfg->beam_photon_plane_cut, 3);
  const double ff = f1 * (1.0 - sc3);
  const double gg = g1 - 27.0 / 16.0 * g2 * cfg->beam_photon_plane_cut + 11.0 / 16.0 * g3 * sc3;
  const double sig_p = sig * (ff + 2.0 * gg);
  const double sig_m = sig_p + 2.0 * sig * gg;
  const double mc_p = ((0.0 + m[0][1]) + m[1][1]) / 4.0;
  const double mc_m = ((0.0 + m[0][2]) + m[1][2]) / 4.0;
  auto incr = [&](int c) {
    const double a = m[0][c] * r->vars[0][c];
    const double b = m[1][c] * r->vars[1][c];
    return std::sqrt(0.0 + (a * a + b * b)) / std::fabs((0.0 + m[0][c]) + m[1][c]);
  };
  const double incr_p = incr(1), incr_m = incr(2);
  line("");
  line("s (pb) :   Sig_cut_Th    Sig_Th      Rapport");
  line("       :   Sig_Num");
  line("       :   Ecart_relatif  Incertitude");
  line("");
  line("s+(pb) : " + fmt_fixed(sig_p, 5) + " | " + fmt_fixed(sig * 3.0, 5) + " | " +
       fmt_fixed(sig_p / (3.0 * sig), 6));
  line("       : " + fmt_fixed(mc_p, 5));
  line("       : " + fmt_fixed(mc_p / sig_p - 1.0, 6) + " | " + fmt_fixed(incr_p, 8) + " | " +
       fmt_fixed((mc_p / sig_p - 1.0) / incr_p, 2));
  line("");
  line("s-(pb) : " + fmt_fixed(sig_m, 5) + " | " + fmt_fixed(sig * 5.0, 4) + " | " +
       fmt_fixed(sig_m / (5.0 * sig), 6));
  line("       : " + fmt_fixed(mc_m, 5));
  line("       : " + fmt_fixed(mc_m / sig_m - 1.0, 6) + " | " + fmt_fixed(incr_m, 9) + " | " +
       fmt_fixed((mc_m / sig_m - 1.0) / incr_m, 2));
  line("");
  return copy_out(s, buf, len);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// K_c(theta) and dK_c/dtheta for theta = (beta+, beta-, M_Z, Gamma_Z) by
// forward-mode dual numbers through the same formulas as above
// (src/coupling.rs:23-33, src/resacc.rs:59-100).
// ---------------------------------------------------------------------------
namespace tp {
namespace {
struct D4 {
  double v;
  double d[4];
};
D4 cst(double x) { return {x, {0, 0, 0, 0}}; }
D4 var(double x, int i) {
  D4 r = cst(x);
  r.d[i] = 1.0;
  return r;
}
D4 operator+(D4 a, D4 b) {
  D4 r{a.v + b.v, {}};
  for (int i = 0; i < 4; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
D4 operator-(D4 a, D4 b) {
  D4 r{a.v - b.v, {}};
  for (int i = 0; i < 4; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
D4 operator*(D4 a, D4 b) {
  D4 r{a.v * b.v, {}};
  for (int i = 0; i < 4; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
D4 operator/(D4 a, D4 b) {
  D4 r{a.v / b.v, {}};
  for (int i = 0; i < 4; ++i) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) / (b.v * b.v);
  return r;
}
}  // namespace
}  // namespace tp

extern "C" int tp_coupling_factors(const tp_config* cfg, double k_out[5], double dk_out[20], double* flux) {
  using namespace tp;
  if (check_config(cfg) || !k_out) return TP_ERR_INVALID;
  const D4 bp = var(cfg->beta_plus, 0), bm = var(cfg->beta_minus, 1);
  const D4 mz = var(cfg->m_z0, 2), gz = var(cfg->g_z0, 3);
  // couplings and the spinor prefactor c1 (theta enters through M_Z only)
  const double e2 = (4.0 * kPi) * cfg->alpha;
  const double e2_z = (4.0 * kPi) * cfg->alpha_z;
  const double cos2w = 1.0 - cfg->sin2_weinberg;
  const D4 mz2 = mz * mz, mz4 = mz2 * mz2;
  const D4 g_beta = cst(-std::sqrt(e2_z / ((4.0 * cos2w) * cfg->sin2_weinberg))) / mz4;
  const double g_a = -powi(std::sqrt(e2), 3);
  EvConst k;
  make_ev_const(*cfg, 0, &k);
  const D4 c1 = cst(k.c1);
  const D4 ga_c1 = cst(g_a) * c1, gb_c1 = g_beta * c1;
  const D4 sc_raw[4] = {ga_c1 * ga_c1, gb_c1 * gb_c1, gb_c1 * gb_c1, cst(-2.0) * cst(g_a) * g_beta * c1 * c1};
  // sigma contributions
  const double fact_com = (1.0 / 6.0) * cfg->gev2_to_picobarn;
  const D4 rw = gz / mz;
  const double p_ab = 1.0 - 4.0 * cfg->sin2_weinberg;
  const double p_bb = p_ab + 8.0 * powi(cfg->sin2_weinberg, 2);
  const D4 c_aa = cst(fact_com * 2.0);
  const D4 c_ab = cst(fact_com * p_ab) / mz2;
  const D4 c_bb = cst(fact_com * p_bb) / mz4;
  const D4 ratio = cst(cfg->e_total) / mz;
  const D4 dzeta = ratio * ratio;
  const D4 delta = (dzeta - cst(1.0)) / rw;
  const D4 prop = cst(1.0) / (cst(1.0) + delta * delta);
  const double norm_weight = event_weight(cfg->e_total) * (std::pow(2.0 * kPi, -5.0) / (double)cfg->num_events);
  const D4 com = cst(norm_weight / 4.0);
  const D4 aa = com * c_aa;
  const D4 bb = com * c_bb * prop / (rw * rw);
  const D4 ab = com * c_ab * cst(2.0) * bp * prop / rw;
  const D4 sc[5] = {aa, bb * bp * bp, bb * bm * bm, ab * delta, cst(0.0) - ab};
  for (int c = 0; c < 5; ++c) {
    const D4 K = sc_raw[c < 3 ? c : 3] * sc[c];
    k_out[c] = K.v;
    if (dk_out)
      for (int i = 0; i < 4; ++i) dk_out[4 * c + i] = K.d[i];
  }
  if (flux) *flux = 1.0 / (2.0 * powi(cfg->e_total, 2));
  return TP_OK;
}
