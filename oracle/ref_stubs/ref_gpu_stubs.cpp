// CPU stand-in for the reference's GPU C-ABI (Born/gpu_funcs_3d.h), linked into
// the oracle's reference library so that the reference's own host classes (rtm_zero_op,
// fd_prop, ...) run end to end on the CPU.  Each entry point keeps the
// reference's module-global state and semantics and runs the propagation
// loops of the oracle (sepx_oracle.c).  Every call is also recorded so tests
// can compare what the reference operator hands to the C-ABI with what the
// product's operator hands to its own.  Test infrastructure only.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../sepx_oracle.h"
#include "param_func.h"
#include "data_rtm_3d.h"
#include "image_rtm_3d.h"
#include "rtm_zero_op_3d.h"
#include "source_func_3d.h"
#include "vel_fd_3d.h"

namespace {
struct CallRec {
  std::string name;
  std::vector<long> iargs;
  std::vector<double> fargs;
};
std::vector<CallRec> g_log;

struct RefState {
  int n_gpus = 1, n1 = 0, n2 = 0, n3 = 0;
  float coeffs[13];
  std::vector<float> damp_tab, vel1, vel2, sinc_s, sinc_d, src_vals, rec_vals;
  std::vector<int> src_loc, rec_loc;
  int nsinc = 8, ns = 0, nd = 0, ntrace = 0, npts_s = 0, rec_nx = 0, rec_ny = 0;
} S;

void rec(const char *name, std::vector<long> i, std::vector<double> f) {
  g_log.push_back(CallRec{name, i, f});
}

orc_ctx ctx() {
  orc_ctx c;
  memset(&c, 0, sizeof(c));
  c.g.n1 = S.n1; c.g.n2 = S.n2; c.g.n3 = S.n3;
  memcpy(c.coeffs, S.coeffs, sizeof(S.coeffs));
  c.damp_tab = S.damp_tab.data(); c.ntab = (int)S.damp_tab.size();
  c.ntrace = S.ntrace; c.nsinc = S.nsinc;
  c.sinc_s = S.sinc_s.data(); c.ns = S.ns;
  c.sinc_d = S.sinc_d.data(); c.nd = S.nd;
  c.nsrc = S.npts_s; c.src_loc = S.src_loc.data(); c.src_vals = S.src_vals.data();
  c.nrec_x = S.rec_nx; c.nrec_y = S.rec_ny; c.rec_loc = S.rec_loc.data();
  return c;
}

// parameters of the drivers' sep_params, read from the stub parameter table
class shim_params : public param_func {
 public:
  virtual int get_int(const char *arg, int def) const {
    int v;
    return getch(arg, "d", &v) ? v : def;
  }
  virtual float get_float(const char *arg, float def) const {
    float v;
    return getch(arg, "f", &v) ? v : def;
  }
};
}  // namespace

extern "C" {

void setup_cuda(int ngpus, int, char **) {
  S.n_gpus = ngpus;
  rec("setup_cuda", {ngpus}, {});
}

void create_gpu_space(float d1, float d2, float d3, float bc_a, float bc_b, float bc_b_y, int n1,
                      int n2, int n3) {
  S.n1 = n1; S.n2 = n2; S.n3 = n3;
  orc_fd_coeffs(d1, d2, d3, S.coeffs);
  int ntab = (n1 > n2 ? (n1 > n3 ? n1 : n3) : (n2 > n3 ? n2 : n3)) / 2 + 1;
  S.damp_tab.assign(ntab, 1.f);
  orc_damp_table_f32(bc_a, bc_b, ntab, S.damp_tab.data());
  S.vel1.assign((size_t)n1 * n2 * n3, 0.f);
  S.vel2.assign((size_t)n1 * n2 * n3, 0.f);
  rec("create_gpu_space", {n1, n2, n3}, {d1, d2, d3, bc_a, bc_b, bc_b_y});
}

void transfer_sinc_table_s(int nsinc, int ns, float **tables) {
  S.nsinc = nsinc; S.ns = ns;
  S.sinc_s.resize((size_t)nsinc * ns);
  for (int i = 0; i < ns; i++) memcpy(&S.sinc_s[(size_t)i * nsinc], tables[i], sizeof(float) * nsinc);
  rec("transfer_sinc_table_s", {nsinc, ns}, {});
}

void transfer_sinc_table_d(int nsinc, int nd, float **tables) {
  S.nd = nd;
  S.sinc_d.resize((size_t)nsinc * nd);
  for (int i = 0; i < nd; i++) memcpy(&S.sinc_d[(size_t)i * nsinc], tables[i], sizeof(float) * nsinc);
  rec("transfer_sinc_table_d", {nsinc, nd}, {});
}

void transfer_source_func(int npts, int nt, int *locs, float *vals) {
  S.npts_s = npts; S.ntrace = nt;
  S.src_loc.assign(locs, locs + npts);
  S.src_vals.assign(vals, vals + (size_t)npts * nt);
  rec("transfer_source_func", {npts, nt}, {});
}

void transfer_receiver_func(int nx, int ny, int nt, int *locs, float *vals) {
  S.rec_nx = nx; S.rec_ny = ny; S.ntrace = nt;
  S.rec_loc.assign(locs, locs + (size_t)nx * ny);
  S.rec_vals.assign(vals, vals + (size_t)nx * ny * nt);
  rec("transfer_receiver_func", {nx, ny, nt}, {});
}

void transfer_vel_func1(int n1, int n2, int n3, float *vel) {
  S.vel1.assign(vel, vel + (size_t)n1 * n2 * n3);
  rec("transfer_vel_func1", {n1, n2, n3}, {});
}

void transfer_vel_func2(int n1, int n2, int n3, float *vel) {
  S.vel2.assign(vel, vel + (size_t)n1 * n2 * n3);
  rec("transfer_vel_func2", {n1, n2, n3}, {});
}

void source_prop(int n1, int n2, int n3, bool damp, bool get_last, float *p0, float *p1, int jt,
                 int npts, int nt) {
  rec("source_prop", {n1, n2, n3, damp, get_last, jt, npts, nt}, {});
  orc_ctx c = ctx();
  std::vector<float> a((size_t)n1 * n2 * n3), b((size_t)n1 * n2 * n3);
  orc_source_prop_f32(&c, S.vel1.data(), a.data(), b.data(), jt, npts, nt);
  if (get_last) {
    memcpy(p0, a.data(), sizeof(float) * a.size());
    memcpy(p1, b.data(), sizeof(float) * b.size());
  }
}

void rtm_forward(int n1, int n2, int n3, int jt, float *img, float *dat, int npts_src, int nt,
                 int nt_big, int nx, int ny) {
  rec("rtm_forward", {n1, n2, n3, jt, npts_src, nt, nt_big, nx, ny}, {});
  orc_ctx c = ctx();
  std::vector<float> buf = S.rec_vals;
  orc_rtm_forward_f32(&c, S.vel1.data(), jt, img, buf.data(), npts_src, nt);
  memcpy(dat, buf.data(), sizeof(float) * (size_t)nt_big * nx * ny);
}

void rtm_adjoint(int n1, int n2, int n3, int jt, float *p0_s, float *p1_s, float *img, int npts,
                 int nt) {
  rec("rtm_adjoint", {n1, n2, n3, jt, npts, nt}, {});
  orc_ctx c = ctx();
  orc_rtm_adjoint_f32(&c, S.vel1.data(), jt, p0_s, p1_s, img, S.rec_vals.data(), npts, nt);
}

// ---- call log ----
void ref_log_clear(void) { g_log.clear(); }
int ref_log_count(void) { return (int)g_log.size(); }
// copies the name (<=63 chars) and up to 16 integer / 8 float arguments
int ref_log_entry(int i, char *name, long *iargs, double *fargs) {
  if (i < 0 || i >= (int)g_log.size()) return -1;
  strncpy(name, g_log[i].name.c_str(), 63);
  name[63] = 0;
  for (size_t k = 0; k < g_log[i].iargs.size() && k < 16; k++) iargs[k] = g_log[i].iargs[k];
  for (size_t k = 0; k < g_log[i].fargs.size() && k < 8; k++) fargs[k] = g_log[i].fargs[k];
  return (int)g_log[i].iargs.size();
}
// last arrays handed to the C-ABI
long ref_last_array(const char *which, void *out, long nbytes) {
  const void *src = nullptr;
  long sz = 0;
  std::string w(which);
  if (w == "vel1") { src = S.vel1.data(); sz = (long)S.vel1.size() * 4; }
  else if (w == "vel2") { src = S.vel2.data(); sz = (long)S.vel2.size() * 4; }
  else if (w == "sinc_s") { src = S.sinc_s.data(); sz = (long)S.sinc_s.size() * 4; }
  else if (w == "sinc_d") { src = S.sinc_d.data(); sz = (long)S.sinc_d.size() * 4; }
  else if (w == "src_loc") { src = S.src_loc.data(); sz = (long)S.src_loc.size() * 4; }
  else if (w == "src_vals") { src = S.src_vals.data(); sz = (long)S.src_vals.size() * 4; }
  else if (w == "rec_loc") { src = S.rec_loc.data(); sz = (long)S.rec_loc.size() * 4; }
  else if (w == "rec_vals") { src = S.rec_vals.data(); sz = (long)S.rec_vals.size() * 4; }
  else return -1;
  if (out && nbytes > 0) memcpy(out, src, (size_t)(sz < nbytes ? sz : nbytes));
  return sz;
}

// ---- the drivers' call sequences (Born/RTM_fwd.cpp, Born/RTM2_3d.cpp) ----
// Inputs are the in-memory files "data", "wavelet", "velocity", "image", "mute"
// and the parameter table; outputs land in "dataout" (forward) or "image"
// (adjoint).
int ref_run_born_forward(void) {
  shim_params pars;
  data_rtm_3d data((char *)"data", &pars);
  source_func wavelet((char *)"wavelet");
  axis asx = data.get_axis(4), asy = data.get_axis(5);
  float src_depth = pars.get_float("src_depth", 0.);
  wavelet.set_sources_3d(src_depth, asx, asy);
  vel_fd_3d vel((char *)"velocity");
  image_rtm_3d image((char *)"image", &vel);
  image.set_source_file(&image);
  oc_float *d2 = new oc_float("dataout", &data);
  data.set_source_file(d2);
  setup_cuda(pars.get_int("n_gpus", 1), 0, 0);
  float aper = pars.get_float("aper", 8.);
  rtm_zero_op op(&pars, &vel, &wavelet, &data, &image, aper, false, false, 0, false);
  op.forward(false, &image, d2, 1);
  delete d2;
  return 0;
}

int ref_run_rtm_adjoint(void) {
  shim_params pars;
  data_rtm_3d data((char *)"data", &pars);
  source_func wavelet((char *)"wavelet");
  float src_depth = pars.get_float("src_depth", 0.);
  vel_fd_3d vel((char *)"velocity");
  image_rtm_3d image((char *)"image", &vel);
  axis asx = data.get_axis(4), asy = data.get_axis(5);
  wavelet.set_sources_3d(src_depth, asx, asy);
  image.zero();
  image.set_source_file(&image);
  oc_float *d2 = new oc_float("dtest.H", &data);
  data.set_source_file(d2);
  setup_cuda(pars.get_int("n_gpus", 1), 0, 0);
  float aper = pars.get_float("aper", 8.);
  rtm_zero_op op(&pars, &vel, &wavelet, &data, &image, aper, false, false, 0, true);
  op.adjoint(false, &image, &data, 1);
  delete d2;
  return 0;
}

}  // extern "C"
