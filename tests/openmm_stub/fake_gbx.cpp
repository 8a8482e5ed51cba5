// A recording stand-in for the gbx C ABI (test infrastructure): lets the
// OpenMM plugin adapter run without a GPU.  Every call appends a line to a
// log the test driver reads; gbx_execute returns a status the driver sets.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gbx.h"

std::vector<std::string> g_log;
gbx_status g_execute_status = GBX_OK;
gbx_config g_last_config;

struct gbx_context {
  int n;
};

namespace {
void log(const std::string& s) { g_log.push_back(s); }
}  // namespace

extern "C" {
const char* gbx_status_string(gbx_status s) { return s == GBX_ERR_STALE_RESULT ? "stale result" : "status"; }
gbx_status gbx_last_error(const gbx_context*, char* buf, size_t len) {
  std::snprintf(buf, len, "an earlier unchecked call lacked the volume terms");
  return GBX_OK;
}
gbx_status gbx_config_preset(int preset, gbx_config* cfg) {
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->model = preset == GBX_PRESET_GBMV1 ? GBX_MODEL_GBMV1 : preset == GBX_PRESET_GBMV2 ? GBX_MODEL_GBMV2 : 0;
  cfg->table_mode = preset == GBX_PRESET_CHARMM_GBSW ? GBX_TABLE_STANDALONE
                    : preset == GBX_PRESET_GBSW_INTEGRAL ? GBX_TABLE_GRID : GBX_TABLE_PERIODIC;
  cfg->alpha0 = -0.180;
  cfg->alpha1 = 1.817;
  log("preset " + std::to_string(preset));
  return GBX_OK;
}
gbx_status gbx_create(const gbx_config* cfg, int n, gbx_context** out) {
  g_last_config = *cfg;
  *out = new gbx_context{n};
  char b[256];
  std::snprintf(b, sizeof(b), "create n=%d model=%d table=%d periodic=%d cutoff=%g box=%g,%g,%g alpha=%g,%g", n,
                cfg->model, cfg->table_mode, cfg->periodic, cfg->cutoff, cfg->box[0], cfg->box[1], cfg->box[2],
                cfg->alpha0, cfg->alpha1);
  log(b);
  return GBX_OK;
}
gbx_status gbx_destroy(gbx_context* c) {
  delete c;
  log("destroy");
  return GBX_OK;
}
gbx_status gbx_set_particle_parameters(gbx_context* c, const double* q, const double* r) {
  char b[128];
  std::snprintf(b, sizeof(b), "params q0=%g r0=%g q%d=%g", q[0], r[0], c->n - 1, q[c->n - 1]);
  log(b);
  return GBX_OK;
}
gbx_status gbx_set_global_parameters(gbx_context*, double a0, double a1) {
  char b[128];
  std::snprintf(b, sizeof(b), "globals %g %g", a0, a1);
  log(b);
  return GBX_OK;
}
gbx_status gbx_create_custom(const gbx_config* cfg, int n, const gbx_custom* cs, gbx_context** out) {
  g_last_config = *cfg;
  *out = new gbx_context{n};
  std::string s = "create_custom n=" + std::to_string(n) + " model=" + std::to_string(cfg->model) + " params";
  for (int k = 0; k < cs->num_params; ++k) s += std::string(" ") + cs->param_names[k];
  s += " integrals";
  for (int k = 0; k < cs->num_integrals; ++k)
    s += std::string(" ") + cs->integral_names[k] + ":" + std::to_string(cs->integral_orders[k]);
  s += " values";
  for (int k = 0; k < cs->num_values; ++k) s += std::string(" ") + cs->value_names[k];
  s += " terms";
  for (int k = 0; k < cs->num_terms; ++k) s += " " + std::to_string(cs->term_types[k]);
  if (cs->num_exclusions > 0) {
    s += " exclusions";
    for (int k = 0; k < cs->num_exclusions; ++k)
      s += " " + std::to_string(cs->exclusions[2 * k]) + "-" + std::to_string(cs->exclusions[2 * k + 1]);
  }
  if (cs->num_param_derivs > 0) {
    s += " param_derivs";
    for (int k = 0; k < cs->num_param_derivs; ++k) s += std::string(" ") + cs->param_deriv_names[k];
  }
  size_t off = 0;
  for (int k = 0; k < cs->num_functions; ++k) {
    char b[160];
    std::snprintf(b, sizeof(b), " function %s n=%d [%g,%g] first=%g last=%g", cs->function_names[k],
                  cs->function_sizes[k], cs->function_ranges[2 * k], cs->function_ranges[2 * k + 1],
                  cs->function_values[off], cs->function_values[off + cs->function_sizes[k] - 1]);
    s += b;
    off += (size_t)cs->function_sizes[k];
  }
  log(s);
  return GBX_OK;
}
gbx_status gbx_get_custom_param_derivs(gbx_context*, double* out, int count) {
  log("param_derivs " + std::to_string(count));
  for (int k = 0; k < count; ++k) out[k] = 0.5 * (k + 1);  // 0.5, 1.0, ...
  return GBX_OK;
}
gbx_status gbx_set_custom_parameters(gbx_context*, const double* p) {
  char b[128];
  std::snprintf(b, sizeof(b), "custom_params p00=%g p01=%g p02=%g", p[0], p[1], p[2]);
  log(b);
  return GBX_OK;
}
gbx_status gbx_set_custom_global(gbx_context*, const char* name, double v) {
  char b[128];
  std::snprintf(b, sizeof(b), "custom_global %s %g", name, v);
  log(b);
  return GBX_OK;
}
gbx_status gbx_set_box(gbx_context*, const double box[3]) {
  char b[128];
  std::snprintf(b, sizeof(b), "box %g %g %g", box[0], box[1], box[2]);
  log(b);
  return GBX_OK;
}
gbx_status gbx_set_atom_order(gbx_context* c, const int* idx) {
  std::string s = "order";
  for (int k = 0; k < c->n; ++k) s += " " + std::to_string(idx[k]);
  log(s);
  return GBX_OK;
}
gbx_status gbx_execute(gbx_context*, const void* posq, unsigned long long* force, int stride, double* energy,
                       int flags, void* stream) {
  char b[160];
  std::snprintf(b, sizeof(b), "execute posq=%lx force=%lx stride=%d energy=%lx flags=%d stream=%lx",
                (unsigned long)(size_t)posq, (unsigned long)(size_t)force, stride, (unsigned long)(size_t)energy,
                flags, (unsigned long)(size_t)stream);
  log(b);
  return g_execute_status;
}
}
