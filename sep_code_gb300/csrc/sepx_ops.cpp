// sepx_ops.cpp -- operator / vector / solver layer on device-resident vectors
// (include/sepx_ops.h).  Host C++ over the C ABI of include/sepx.h: every
// vector lives in HBM, BLAS-1 and FP64 dots run on the GPU, the per-shot
// set-up follows rtm_zero_op (Born/rtm_zero_op_3d.cpp) with in-memory inputs.
#include "../../include/sepx_ops.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/sepx.h"
#include "../../include/sepx_host.h"
#include "sepx_common.h"

namespace {

void ck(int rc, const char *what) {
  if (rc != 0) throw std::runtime_error(std::string(what) + ": " + sepx_last_error());
}

unsigned long long g_random_seed = 0x5EB0C0DE2026ull;

hypercube_float *hf(my_vector *v) {
  auto *h = dynamic_cast<hypercube_float *>(v);
  if (!h) throw std::runtime_error("expected a hypercube_float");
  return h;
}

super_vector *sv(my_vector *v) {
  auto *s = dynamic_cast<super_vector *>(v);
  if (!s) throw std::runtime_error("expected a super_vector");
  return s;
}

}  // namespace

// ------------------------------------------------------------------ my_vector
my_vector *my_vector::clone_zero() {
  my_vector *v = clone_vec();
  v->zero();
  return v;
}

// ------------------------------------------------------------------ hypercube_float
hypercube_float::hypercube_float(const std::vector<axis> &ax) : axes(ax) {
  name = "hypercube_float";
  n123 = 1;
  for (const auto &a : axes) n123 *= a.n;
  // the first device vector brings up the GPU (setup_cuda(1) does nothing
  // once it has run), so vectors may be built before the program's own
  // setup_cuda call, as the reference's programs build theirs
  ck(sepx_setup_cuda(1), "setup_cuda");
  ck(sepx_vec_alloc(&vals, n123), "hypercube_float alloc");
  ck(sepx_vec_fill(vals, n123, 0.f), "hypercube_float fill");
}

hypercube_float::~hypercube_float() { sepx_vec_free(vals); }

my_vector *hypercube_float::clone_vec() {
  auto *h = new hypercube_float(axes);
  ck(sepx_vec_copy(h->vals, vals, n123), "clone_vec");
  return h;
}

my_vector *hypercube_float::clone_space() { return new hypercube_float(axes); }

void hypercube_float::scale(double num) { ck(sepx_vec_scale(vals, n123, num), "scale"); }

void hypercube_float::scale_add(double mes, my_vector *vec, double other) {
  ck(sepx_vec_scale_add(vals, hf(vec)->vals, n123, mes, other), "scale_add");
}

void hypercube_float::scale_add(double sc1, my_vector *v1, double sc2, my_vector *v2) {
  ck(sepx_vec_scale_add2(vals, hf(v1)->vals, hf(v2)->vals, n123, sc1, sc2), "scale_add");
}

void hypercube_float::set_val(double val) { ck(sepx_vec_fill(vals, n123, (float)val), "set_val"); }

void hypercube_float::add(my_vector *vec) { ck(sepx_vec_add(vals, hf(vec)->vals, n123), "add"); }

void hypercube_float::mult(my_vector *vec) { ck(sepx_vec_mult(vals, hf(vec)->vals, n123), "mult"); }

double hypercube_float::sum() {
  double r = 0;
  ck(sepx_dot_f32(vals, nullptr, n123, &r), "sum");
  return r;
}

double hypercube_float::dot(my_vector *vec) {
  double r = 0;
  ck(sepx_dot_f32(vals, hf(vec)->vals, n123, &r), "dot");
  return r;
}

void hypercube_float::random() { ck(sepx_vec_random(vals, n123, g_random_seed++), "random"); }

bool hypercube_float::check_match(const my_vector *v2) const {
  auto *o = dynamic_cast<const hypercube_float *>(v2);
  return o && o->n123 == n123;
}

void hypercube_float::upload(const float *host) { ck(sepx_vec_upload(vals, host, n123), "upload"); }

void hypercube_float::download(float *host) const {
  ck(sepx_vec_download(host, vals, n123), "download");
}

// ------------------------------------------------------------------ super_vector
super_vector::super_vector(const std::vector<my_vector *> &vs, bool just_space) {
  name = "super_vector";
  for (auto *v : vs) vecs.push_back(just_space ? v->clone_space() : v->clone_vec());
}

super_vector::~super_vector() {
  for (auto *v : vecs) delete v;
}

my_vector *super_vector::clone_vec() { return new super_vector(vecs, false); }
my_vector *super_vector::clone_space() { return new super_vector(vecs, true); }
void super_vector::scale(double num) {
  for (auto *v : vecs) v->scale(num);
}
void super_vector::scale_add(double mes, my_vector *vec, double other) {
  auto *o = sv(vec);
  for (size_t i = 0; i < vecs.size(); i++) vecs[i]->scale_add(mes, o->vecs[i], other);
}
void super_vector::scale_add(double sc1, my_vector *v1, double sc2, my_vector *v2) {
  auto *a = sv(v1), *b = sv(v2);
  for (size_t i = 0; i < vecs.size(); i++) vecs[i]->scale_add(sc1, a->vecs[i], sc2, b->vecs[i]);
}
void super_vector::set_val(double val) {
  for (auto *v : vecs) v->set_val(val);
}
void super_vector::add(my_vector *vec) {
  auto *o = sv(vec);
  for (size_t i = 0; i < vecs.size(); i++) vecs[i]->add(o->vecs[i]);
}
void super_vector::mult(my_vector *vec) {
  auto *o = sv(vec);
  for (size_t i = 0; i < vecs.size(); i++) vecs[i]->mult(o->vecs[i]);
}
double super_vector::sum() {
  double s = 0;
  for (auto *v : vecs) s += v->sum();
  return s;
}
double super_vector::dot(my_vector *vec) {
  auto *o = sv(vec);
  double s = 0;
  for (size_t i = 0; i < vecs.size(); i++) s += vecs[i]->dot(o->vecs[i]);
  return s;
}
void super_vector::random() {
  for (auto *v : vecs) v->random();
}
bool super_vector::check_match(const my_vector *v2) const {
  auto *o = dynamic_cast<const super_vector *>(v2);
  if (!o || o->vecs.size() != vecs.size()) return false;
  for (size_t i = 0; i < vecs.size(); i++)
    if (!vecs[i]->check_match(o->vecs[i])) return false;
  return true;
}

// ------------------------------------------------------------------ operators
my_operator::~my_operator() {
  delete domain;
  delete range;
}

void my_operator::set_domain(my_vector *dom) {
  delete domain;
  domain = dom->clone_space();
}

void my_operator::set_range(my_vector *ran) {
  delete range;
  range = ran->clone_space();
}

void my_operator::hessian(my_vector *in, my_vector *out) {
  std::unique_ptr<my_vector> d(range->clone_vec());
  forward(false, in, d.get());
  adjoint(false, out, d.get());
}

// Born/my_operator.cpp:14-76
bool my_operator::dot_test(bool verb, double *out, double tol) {
  std::unique_ptr<my_vector> mod1(domain->clone_vec()), mod2(domain->clone_vec());
  std::unique_ptr<my_vector> dat1(range->clone_vec()), dat2(range->clone_vec());
  mod1->random();
  dat2->random();
  forward(false, mod1.get(), dat1.get());
  const double dot1 = dat1->dot(dat2.get());
  adjoint(false, mod2.get(), dat2.get());
  const double dot2 = mod2->dot(mod1.get());
  if (verb) fprintf(stderr, "Dot(add=false) %g %g\n", dot1, dot2);
  forward(true, mod1.get(), dat1.get());
  adjoint(true, mod2.get(), dat2.get());
  const double dot3 = mod1->dot(mod2.get());
  const double dot4 = dat1->dot(dat2.get());
  if (verb) fprintf(stderr, "Dot(add=true) %g %g\n", dot4, dot3);
  if (out) {
    out[0] = dot1; out[1] = dot2; out[2] = dot3; out[3] = dot4;
  }
  if (std::fabs(dot1) < 1e-12 || std::fabs(dot3) < 1e-12) return false;
  if (std::fabs((dot1 - dot2) / dot1) > tol) return false;
  if (std::fabs((dot3 - dot4) / dot3) > tol) return false;
  return true;
}

i_op::i_op(my_vector *mod, my_vector *dat) {
  set_domain(mod);
  set_range(dat);
}
bool i_op::forward(bool add, my_vector *model, my_vector *data, int) {
  data->scale_add(add ? 1.0 : 0.0, model, scale);
  return true;
}
bool i_op::adjoint(bool add, my_vector *model, my_vector *data, int) {
  model->scale_add(add ? 1.0 : 0.0, data, scale);
  return true;
}

row_op::row_op(const std::vector<my_operator *> &os) : ops(os) {
  domain = ops.front()->domain->clone_space();
  range = ops.back()->range->clone_space();
}
row_op::~row_op() {}
bool row_op::forward(bool add, my_vector *model, my_vector *data, int iter) {
  my_vector *dom = model;
  for (size_t i = 0; i < ops.size(); i++) {
    const bool last = (i + 1 == ops.size());
    my_vector *ran = last ? data : ops[i]->range->clone_zero();
    if (!ops[i]->forward(last ? add : false, dom, ran, iter)) return false;
    if (i != 0) delete dom;
    dom = ran;
  }
  return true;
}
bool row_op::adjoint(bool add, my_vector *model, my_vector *data, int iter) {
  my_vector *ran = data;
  for (int i = (int)ops.size() - 1; i >= 0; i--) {
    my_vector *dom = (i != 0) ? ops[i]->domain->clone_zero() : model;
    if (!ops[i]->adjoint(i != 0 ? false : add, dom, ran, iter)) return false;
    if (i != (int)ops.size() - 1) delete ran;
    ran = dom;
  }
  return true;
}

col_op::col_op(const std::vector<my_operator *> &os) : ops(os) {
  std::vector<my_vector *> rs;
  for (auto *o : ops) rs.push_back(o->range);
  range = new super_vector(rs, true);
  domain = ops.front()->domain->clone_space();
}
bool col_op::forward(bool add, my_vector *model, my_vector *data, int iter) {
  auto *d = sv(data);
  for (size_t i = 0; i < ops.size(); i++)
    if (!ops[i]->forward(add, model, d->vecs[i], iter)) return false;
  return true;
}
bool col_op::adjoint(bool add, my_vector *model, my_vector *data, int iter) {
  auto *d = sv(data);
  bool a = add;
  for (size_t i = 0; i < ops.size(); i++) {
    if (!ops[i]->adjoint(a, model, d->vecs[i], iter)) return false;
    a = true;
  }
  return true;
}

// ------------------------------------------------------------------ cgstep (Born/cgstep.cpp)
cgstep::~cgstep() {
  delete s;
  delete ss;
}
void cgstep::alloc_step(my_vector *mod, my_vector *dat) {
  delete s;
  delete ss;
  s = mod->clone_vec();
  ss = dat->clone_vec();
  forget_it();
}
void cgstep::forget_it() {
  forget = true;
  s->zero();
  ss->zero();
  small = 1e-20;
}
bool cgstep::step_it(int, my_vector *m, my_vector *g, my_vector *rr, my_vector *gg, double *vv) {
  double alfa, beta;
  if (forget) {
    beta = 0;
    const double gg_gg = gg->dot(gg);
    if (std::fabs(gg_gg) < small) return false;
    alfa = -gg->dot(rr) / gg_gg;
  } else {
    const double gg_gg = gg->dot(gg), ss_ss = ss->dot(ss), gg_ss = gg->dot(ss);
    if (std::fabs(gg_gg) < small || std::fabs(ss_ss) < small) return false;
    const double determ = gg_gg * ss_ss * (1.0 - gg_ss / gg_gg * gg_ss / ss_ss);
    const double gg_rr = -gg->dot(rr), ss_rr = -ss->dot(rr);
    alfa = (ss_ss * gg_rr - gg_ss * ss_rr) / determ;
    beta = (-gg_ss * gg_rr + gg_gg * ss_rr) / determ;
  }
  s->scale_add(beta, g, alfa);
  ss->scale_add(beta, gg, alfa);
  m->add(s);
  rr->add(ss);
  *vv = rr->dot(rr);
  forget = false;
  return true;
}

// ------------------------------------------------------------------ solvers (Born/lin_solver.cpp)
lin_solver::~lin_solver() {
  delete rr;
  delete m;
  delete gg;
  delete g;
  if (own_oper) delete oper;
}
void lin_solver::init_solve(step *s) { st = s; }
void lin_solver::create_solver_vecs() {
  gg = rr->clone_zero();
  m = oper->domain->clone_zero();
  g = oper->domain->clone_zero();
  st->alloc_step(m, rr);
}
my_vector *lin_solver::init_rr(my_vector *data, my_operator *op, my_vector *m0) {
  my_vector *r = data->clone_vec();
  r->scale(-1.);
  if (m0) op->forward(true, m0, r);
  return r;
}
bool lin_solver::solve(int niter) {
  const auto t0 = std::chrono::steady_clock::now();
  double prev = rr->dot(rr);
  const double rr0 = prev;
  bool use_dir = dir != nullptr;
  if (dir_policy == SEPX_DIR_ADAPTIVE && probe_every < 1)
    throw std::runtime_error("probe_every must be at least 1");
  double gain_plain = -1.0;   // fraction of rr.rr removed by the latest plain step
  int plain_run = 0;
  for (int iter = 0; iter < niter; iter++) {
    oper->adjoint(false, g, rr, iter);
    if (use_dir) {
      auto *gh = dynamic_cast<hypercube_float *>(g);
      if (!gh) throw std::runtime_error("direction preconditioning needs a hypercube_float model");
      ck(dir(dir_ctx, gh->vals, gh->n123), "direction preconditioner");
    }
    oper->forward(false, g, gg, iter);
    double val = 0;
    const bool valid = st->step_it(iter, m, g, rr, gg, &val);
    if (!valid) return false;
    used_dir.push_back(use_dir ? 1 : 0);
    const double gain = prev > 0 ? 1.0 - val / prev : 0.0;
    bool next = use_dir;
    if (dir != nullptr && dir_policy == SEPX_DIR_ADAPTIVE) {
      if (use_dir) {
        // keep the preconditioned direction while it removes at least the
        // fraction the latest plain step removed
        next = gain_plain < 0 ? !(fallback_ratio > 0 && val > fallback_ratio * prev)
                              : gain >= gain_plain;
        plain_run = 0;
      } else {
        gain_plain = gain;
        next = ++plain_run >= probe_every;
      }
    } else if (use_dir && fallback_ratio > 0 && val > fallback_ratio * prev) {
      // plain CG is the fallback: once a preconditioned step lowers rr.rr by
      // less than the ratio allows, the remaining iterations use plain g
      next = false;
    }
    if (use_dir && !next && fallback_iter < 0) fallback_iter = iter;
    use_dir = next;
    prev = val;
    resid.push_back(val);
    seconds.push_back(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    if (verb > 0) fprintf(stderr, "iter %d residual %g\n", iter, val);
    if (target > 0 && val <= target * target * rr0) break;
  }
  return true;
}

simple_solver::simple_solver(step *s, my_vector *data, my_operator *op, my_vector *m0) {
  init_solve(s);
  rr = init_rr(data, op, m0);
  oper = op;
  create_solver_vecs();
}

prec_solver::prec_solver(step *s, my_vector *data, my_operator *op, my_operator *prec, float eps,
                         my_vector *m0) {
  init_solve(s);
  my_vector *rtemp = init_rr(data, op, m0);
  std::unique_ptr<my_vector> pdom(prec->domain->clone_zero());
  iop = new i_op(pdom.get(), pdom.get());
  iop->set_scale(eps);
  chain = new row_op({prec, op});
  oper = new col_op({chain, iop});
  own_oper = true;
  rr = new super_vector({rtemp, pdom.get()}, false);
  delete rtemp;
  pop = prec;
  create_solver_vecs();
}
prec_solver::~prec_solver() {
  delete chain;
  delete iop;
}
my_vector *prec_solver::return_model() {
  my_vector *mod = pop->range->clone_zero();
  pop->forward(false, m, mod);
  return mod;
}

reg_solver::reg_solver(step *s, my_vector *data, my_operator *op, my_operator *reg, float eps,
                       my_vector *m0) {
  init_solve(s);
  my_vector *rtemp = init_rr(data, op, m0);
  std::unique_ptr<my_vector> rdom(reg->range->clone_zero());
  reg->set_scale(eps);
  oper = new col_op({op, reg});
  own_oper = true;
  rr = new super_vector({rtemp, rdom.get()}, false);
  delete rtemp;
  create_solver_vecs();
}

// ------------------------------------------------------------------ rtm_zero_op
struct rtm_zero_op::shot_setup {
  bool ready = false;
  std::vector<int> src_locs, rec_locs;
  std::vector<float> vals8, vals9, vrand, sf_p0, sf_p1;
};

struct rtm_zero_op::impl {
  sepx_rtm_problem p;
  std::vector<float> vel, wavelet_deriv, shot_xyz;
  int n1 = 0, n2 = 0, n3 = 0;
  float o[3] = {0, 0, 0}, d[3] = {1, 1, 1};
  float dt = 0;
  int nt = 0, jts = 1, jtd = 1, nt_big = 0, nrec = 0;
  int f[3] = {0, 0, 0};
  std::vector<float> sinc_s, sinc_d;
  std::vector<shot_setup> shots;
  bool fields_ready = false;
  bool verb = false;   // progress lines on stderr
  bool redo = false;   // propagate the source wavefields again at every adjoint

  void upload_tables() {
    std::vector<float *> rs(jts), rd(jtd);
    for (int i = 0; i < jts; i++) rs[i] = sinc_s.data() + (size_t)i * 8;
    for (int i = 0; i < jtd; i++) rd[i] = sinc_d.data() + (size_t)i * 8;
    ck(sepx_transfer_sinc_table_s(8, jts, rs.data()), "transfer_sinc_table_s");
    ck(sepx_transfer_sinc_table_d(8, jtd, rd.data()), "transfer_sinc_table_d");
  }

  shot_setup &shot(int is) {
    shot_setup &s = shots[is];
    if (s.ready) return s;
    const float sx = shot_xyz[3 * is], sy = shot_xyz[3 * is + 1], sz = shot_xyz[3 * is + 2];
    s.src_locs.resize(9);
    s.vals8.resize((size_t)9 * nt_big);
    s.vals9.resize((size_t)9 * (nt_big + 1));
    std::vector<int> l9(9);
    sepx_host_source_func(wavelet_deriv.data(), (int)wavelet_deriv.size(), sx, sy, sz, n1, n2, o[0],
                          o[1], o[2], d[0], d[1], d[2], nt_big, s.src_locs.data(), s.vals8.data());
    sepx_host_source_func(wavelet_deriv.data(), (int)wavelet_deriv.size(), sx, sy, sz, n1, n2, o[0],
                          o[1], o[2], d[0], d[1], d[2], nt_big + 1, l9.data(), s.vals9.data());
    const int seed = s.src_locs[3] - (s.src_locs[3] / 10000) * 10000;
    s.vrand.resize((size_t)n1 * n2 * n3);
    sepx_host_rand_subspace(seed, p.nbound, p.nbound, p.nbound, dt, vel.data(), p.m1, p.m2, p.m3, p.mo1,
                            p.mo2, p.mo3, p.d1, p.d2, p.d3, n1, n2, n3, o[0], o[1], o[2], d[0], d[1],
                            d[2], s.vrand.data());
    s.rec_locs.resize(nrec);
    sepx_host_receiver_map(p.rnx, p.rny, p.ro2, p.rd2, p.ro3, p.rd3, p.rec_depth, n1, n2, o[0],
                           o[1], o[2], d[0], d[1], d[2], s.rec_locs.data());
    s.ready = true;
    return s;
  }
};

rtm_zero_op::rtm_zero_op(const sepx_rtm_problem &p) : d(new impl) {
  init(p);
  if (p.mode == 0) create_source_fields();
}

// Born/rtm_zero_op_3d.cpp:8-36 with fd_prop::set_fd_basics
// (Born/fd_prop_3d.cpp:35-55): parameters bc_a, bc_b, nbound; receiver depth
// rec_depth; the padded grid, stability, sinc tables and device grid.
rtm_zero_op::rtm_zero_op(param_func *par, vel_fd_3d *vel, source_func *source, data_rtm_3d *data,
                         image_rtm_3d *image, float /*aper*/, bool verb, bool /*encode*/,
                         int * /*rand_vec*/, bool do_src, bool redo_src)
    : d(new impl) {
  if (!par || !vel || !source || !data || !image)
    throw std::runtime_error("rtm_zero_op: NULL argument");
  if (vel->axes.size() != 3) throw std::runtime_error("rtm_zero_op: the velocity needs three axes");
  if (data->axes.size() < 3)
    throw std::runtime_error("rtm_zero_op: the data needs (t, x, y[, shots]) axes");
  const int nshots = data->nshots();
  if ((int)source->sx.size() != nshots)
    throw std::runtime_error("rtm_zero_op: " + std::to_string(source->sx.size()) +
                             " source positions for " + std::to_string(nshots) + " shots of data");
  for (int k = 1; k <= 3; k++) {
    const axis a = image->get_axis(k), v = vel->get_axis(k);
    if (a.n != v.n || a.o != v.o || a.d != v.d)
      throw std::runtime_error("rtm_zero_op: the image grid differs from the velocity grid");
  }
  std::vector<float> xyz(3 * (size_t)nshots);
  for (int i = 0; i < nshots; i++) {
    xyz[3 * i] = source->sx[i];
    xyz[3 * i + 1] = source->sy[i];
    xyz[3 * i + 2] = source->sz[i];
  }
  sepx_rtm_problem p;
  std::memset(&p, 0, sizeof p);
  p.vel = vel->vals.data();
  p.m1 = vel->axes[0].n; p.m2 = vel->axes[1].n; p.m3 = vel->axes[2].n;
  p.d1 = vel->axes[0].d; p.d2 = vel->axes[1].d; p.d3 = vel->axes[2].d;
  p.mo1 = vel->axes[0].o; p.mo2 = vel->axes[1].o; p.mo3 = vel->axes[2].o;
  p.wavelet = source->wavelet.data();
  p.nwav = (int)source->wavelet.size();
  p.dtw = source->get_dt();
  p.data_nt = data->axes[0].n;
  p.data_dt = data->axes[0].d;
  p.rnx = data->axes[1].n; p.ro2 = data->axes[1].o; p.rd2 = data->axes[1].d;
  p.rny = data->axes[2].n; p.ro3 = data->axes[2].o; p.rd3 = data->axes[2].d;
  p.rec_depth = par->get_float("rec_depth", data->sz);
  p.nshots = nshots;
  p.shot_xyz = xyz.data();
  p.bc_a = par->get_float("bc_a", 50.f);
  p.bc_b = par->get_float("bc_b", .0005f);
  p.nbound = par->get_int("nbound", (int)p.bc_a);
  p.mode = 0;
  init(p);
  d->verb = verb;
  d->redo = redo_src;
  if (do_src && !redo_src) create_source_fields();
}

void rtm_zero_op::init(const sepx_rtm_problem &p) {
  impl &I = *d;
  I.p = p;
  const long long nm = (long long)p.m1 * p.m2 * p.m3;
  I.vel.assign(p.vel, p.vel + nm);
  std::vector<float> w(p.wavelet, p.wavelet + p.nwav);
  I.wavelet_deriv.resize(p.nwav);
  sepx_host_wavelet_deriv(w.data(), p.nwav, p.dtw, I.wavelet_deriv.data());
  I.shot_xyz.assign(p.shot_xyz, p.shot_xyz + 3 * p.nshots);
  // the caller's arrays are copied: keep no pointer to them
  I.p.vel = I.vel.data();
  I.p.wavelet = nullptr;
  I.p.shot_xyz = I.shot_xyz.data();
  // fd_prop::calc_stability (Born/fd_prop_3d.cpp:7-26) with vel_fd_3d's
  // get_min_samp (it returns dz when dy < dx, Born/vel_fd_3d.h:17)
  double vmax = I.vel[0];
  for (float v : I.vel) vmax = std::max(vmax, (double)v);
  const float dx = p.d1, dy = p.d2, dz = p.d3;
  const float dmin = (dz < dx && dz < dy) ? dz : ((dy < dx) ? dz : dx);
  I.dt = sepx_host_calc_stability((float)vmax, dmin, p.data_dt, p.data_nt, &I.nt);
  const float rem = p.dtw / I.dt - (int)(p.dtw / I.dt + .001);
  if (std::fabs(rem) > .01) throw std::runtime_error("wavelet and propagation sampling do not match");
  I.jts = (int)(p.dtw / I.dt);
  I.jtd = (int)(p.data_dt / I.dt);
  if (I.jts < 1 || I.jtd < 1) throw std::runtime_error("invalid time ratios");
  I.nt_big = 8 + p.data_nt;
  I.nrec = p.rnx * p.rny;
  sepx_host_compute_size(p.m1, p.m2, p.m3, p.nbound, p.nbound, p.nbound, 4, &I.n1, &I.n2, &I.n3);
  const int nb = p.nbound + 4;
  I.d[0] = p.d1; I.d[1] = p.d2; I.d[2] = p.d3;
  const float mo[3] = {p.mo1, p.mo2, p.mo3};
  for (int k = 0; k < 3; k++) {
    I.o[k] = -I.d[k] * (float)nb;
    // image_rtm_3d::extract_sub (Born/image_rtm_3d.cpp:52-90): model index =
    // padded index + f, f = (int)((o_padded - o_model) / d_model)
    I.f[k] = (int)((I.o[k] - mo[k]) / I.d[k]);
  }
  I.sinc_s.resize((size_t)I.jts * 8);
  I.sinc_d.resize((size_t)I.jtd * 8);
  sepx_host_sinc_table(I.jts, 8, I.sinc_s.data());
  sepx_host_sinc_table(I.jtd, 8, I.sinc_d.data());
  ck(sepx_setup_cuda(1), "setup_cuda");
  ck(sepx_create_gpu_space(p.d1, p.d2, p.d3, p.bc_a, p.bc_b, p.bc_b, I.n1, I.n2, I.n3),
     "create_gpu_space");
  I.upload_tables();
  I.shots.resize(p.nshots);
  std::unique_ptr<hypercube_float> m0(new_model()), d0(new_data());
  set_domain(m0.get());
  set_range(d0.get());
}

rtm_zero_op::~rtm_zero_op() { delete d; }

hypercube_float *rtm_zero_op::new_model() const {
  return new hypercube_float({axis(d->p.m1, d->p.mo1, d->p.d1), axis(d->p.m2, d->p.mo2, d->p.d2),
                              axis(d->p.m3, d->p.mo3, d->p.d3)});
}

hypercube_float *rtm_zero_op::new_data() const {
  return new hypercube_float({axis(d->p.data_nt, 0.f, d->p.data_dt), axis(d->p.rnx, d->p.ro2, d->p.rd2),
                              axis(d->p.rny, d->p.ro3, d->p.rd3), axis(d->p.nshots)});
}

// Born/rtm_zero_op_3d.cpp:38-85: the last two source wavefields of every shot
void rtm_zero_op::create_source_fields() {
  impl &I = *d;
  const size_t nv = (size_t)I.n1 * I.n2 * I.n3;
  for (int is = 0; is < I.p.nshots; is++) {
    shot_setup &s = I.shot(is);
    ck(sepx_transfer_source_func(9, I.nt_big + 1, s.src_locs.data(), s.vals9.data()),
       "transfer_source_func");
    ck(sepx_transfer_vel_func1(I.n1, I.n2, I.n3, s.vrand.data()), "transfer_vel_func1");
    s.sf_p0.resize(nv);
    s.sf_p1.resize(nv);
    ck(sepx_source_prop(I.n1, I.n2, I.n3, false, true, s.sf_p0.data(), s.sf_p1.data(), I.jts, 9,
                        I.nt),
       "source_prop");
  }
  I.fields_ready = true;
}

// Born/rtm_zero_op_3d.cpp:87-183
bool rtm_zero_op::forward(bool add, my_vector *model, my_vector *data, int) {
  impl &I = *d;
  auto *m = hf(model), *dv = hf(data);
  if (!add) dv->zero();
  const long long slab = (long long)I.nrec * I.p.data_nt;
  for (int is = 0; is < I.p.nshots; is++) {
    if (I.verb) fprintf(stderr, "Forward shot %d of %d\n", is, I.p.nshots);
    shot_setup &s = I.shot(is);
    ck(sepx_transfer_source_func(9, I.nt_big, s.src_locs.data(), s.vals8.data()), "transfer_source_func");
    ck(sepx_transfer_vel_func1(I.n1, I.n2, I.n3, s.vrand.data()), "transfer_vel_func1");
    ck(sepx_set_receivers(I.p.rnx, I.p.rny, I.nt_big, s.rec_locs.data()), "set_receivers");
    ck(sepx_op_image_to_padded(m->vals, I.p.m1, I.p.m2, I.p.m3, I.f[0], I.f[1], I.f[2]),
       "image_to_padded");
    if (I.p.mode == 0)
      ck(sepx_rtm_forward_resident(I.jtd, 9, I.nt), "rtm_forward");
    else
      ck(sepx_lin_forward_resident(I.jtd, 9, I.nt, I.p.snap_js, I.p.snap_prec), "lin_forward");
    ck(sepx_op_traces_to_data(dv->vals + is * slab, I.p.data_nt, I.p.data_dt), "traces_to_data");
  }
  ck(sepx_synchronize(), "synchronize");
  return true;
}

// Born/rtm_zero_op_3d.cpp:185-293
bool rtm_zero_op::adjoint(bool add, my_vector *model, my_vector *data, int) {
  impl &I = *d;
  if (I.redo && I.p.mode == 0) create_source_fields();
  auto *m = hf(model), *dv = hf(data);
  if (!add) m->zero();
  const long long slab = (long long)I.nrec * I.p.data_nt;
  for (int is = 0; is < I.p.nshots; is++) {
    if (I.verb) fprintf(stderr, "Adjoint shot %d of %d\n", is, I.p.nshots);
    shot_setup &s = I.shot(is);
    ck(sepx_transfer_source_func(9, I.nt_big, s.src_locs.data(), s.vals8.data()), "transfer_source_func");
    ck(sepx_transfer_vel_func1(I.n1, I.n2, I.n3, s.vrand.data()), "transfer_vel_func1");
    ck(sepx_set_receivers(I.p.rnx, I.p.rny, I.nt_big, s.rec_locs.data()), "set_receivers");
    ck(sepx_op_data_to_traces(dv->vals + is * slab, I.p.data_nt, I.p.data_dt), "data_to_traces");
    if (I.p.mode == 0) {
      if (!I.fields_ready) create_source_fields();
      // the stored fields are read back swapped (:254-262): newest as p0_s
      ck(sepx_set_source_fields(s.sf_p1.data(), s.sf_p0.data()), "set_source_fields");
      ck(sepx_rtm_adjoint_resident(I.jtd, 9, I.nt, 0), "rtm_adjoint");
    } else {
      ck(sepx_lin_source_pass(I.jtd, 9, I.nt, I.p.snap_js, I.p.snap_prec), "lin_source_pass");
      ck(sepx_lin_adjoint_resident(I.jtd, I.nt, I.p.snap_js, I.p.snap_prec), "lin_adjoint");
    }
    ck(sepx_op_padded_to_image(m->vals, I.p.m1, I.p.m2, I.p.m3, I.f[0], I.f[1], I.f[2]),
       "padded_to_image");
  }
  ck(sepx_synchronize(), "synchronize");
  return true;
}

// ------------------------------------------------------------------ C API
namespace {
struct op_box {
  std::unique_ptr<rtm_zero_op> op;
  std::unique_ptr<hypercube_float> model, data;
};
}  // namespace

extern "C" {

sepx_op_handle sepx_rtm_op_create(const sepx_rtm_problem *p) {
  try {
    if (!p) {
      sepx::set_error("rtm_zero_op: problem is NULL");
      return nullptr;
    }
    std::unique_ptr<op_box> b(new op_box);
    b->op.reset(new rtm_zero_op(*p));
    b->model.reset(b->op->new_model());
    b->data.reset(b->op->new_data());
    return b.release();
  } catch (const std::exception &e) {
    sepx::set_error("rtm_zero_op: %s", e.what());
    return nullptr;
  }
}

void sepx_rtm_op_destroy(sepx_op_handle h) { delete static_cast<op_box *>(h); }

long long sepx_rtm_op_model_size(sepx_op_handle h) {
  if (!h) return sepx::set_error("model_size: NULL operator");
  return static_cast<op_box *>(h)->model->n123;
}

long long sepx_rtm_op_data_size(sepx_op_handle h) {
  if (!h) return sepx::set_error("data_size: NULL operator");
  return static_cast<op_box *>(h)->data->n123;
}

int sepx_rtm_op_forward(sepx_op_handle h, int add, const float *model, float *data) {
  try {
    if (!h || !model || !data) return sepx::set_error("forward: NULL argument");
    auto *b = static_cast<op_box *>(h);
    b->model->upload(model);
    if (add) b->data->upload(data);
    b->op->forward(add != 0, b->model.get(), b->data.get());
    b->data->download(data);
    return 0;
  } catch (const std::exception &e) {
    return sepx::set_error("forward: %s", e.what());
  }
}

int sepx_rtm_op_adjoint(sepx_op_handle h, int add, float *model, const float *data) {
  try {
    if (!h || !model || !data) return sepx::set_error("adjoint: NULL argument");
    auto *b = static_cast<op_box *>(h);
    b->data->upload(data);
    if (add) b->model->upload(model);
    b->op->adjoint(add != 0, b->model.get(), b->data.get());
    b->model->download(model);
    return 0;
  } catch (const std::exception &e) {
    return sepx::set_error("adjoint: %s", e.what());
  }
}

int sepx_rtm_op_dot_test(sepx_op_handle h, unsigned long long seed, double out[4]) {
  try {
    if (!h || !out) return sepx::set_error("dot_test: NULL argument");
    g_random_seed = seed;
    static_cast<op_box *>(h)->op->dot_test(false, out);
    return 0;
  } catch (const std::exception &e) {
    return sepx::set_error("dot_test: %s", e.what());
  }
}

int sepx_lsrtm(sepx_op_handle h, const float *data, int niter, float *model, double *resid,
               double *seconds, sepx_direction_fn dir, void *dir_ctx, double fallback_ratio,
               int *fallback_iter) {
  try {
    if (!h || !data || !model) return sepx::set_error("lsrtm: NULL argument");
    if (niter < 0) return sepx::set_error("lsrtm: niter %d < 0", niter);
    auto *b = static_cast<op_box *>(h);
    b->data->upload(data);
    cgstep st;
    simple_solver solv(&st, b->data.get(), b->op.get());
    solv.dir = dir;
    solv.dir_ctx = dir_ctx;
    solv.fallback_ratio = fallback_ratio;
    solv.solve(niter);
    if (fallback_iter) *fallback_iter = solv.fallback_iter;
    std::unique_ptr<my_vector> mod(solv.return_model());
    hf(mod.get())->download(model);
    for (size_t i = 0; i < solv.resid.size(); i++) {
      if (resid) resid[i] = solv.resid[i];
      if (seconds) seconds[i] = solv.seconds[i];
    }
    for (size_t i = solv.resid.size(); i < (size_t)niter; i++) {
      if (resid) resid[i] = -1.0;
      if (seconds) seconds[i] = -1.0;
    }
    return 0;
  } catch (const std::exception &e) {
    return sepx::set_error("lsrtm: %s", e.what());
  }
}

int sepx_lsrtm_ex(sepx_op_handle h, const float *data, int niter, const sepx_lsrtm_opts *opts,
                  float *model, double *resid, double *seconds, int *used_dir, int *iters_done) {
  try {
    if (!opts) return sepx::set_error("lsrtm_ex: opts is NULL");
    if (!h || !data || !model) return sepx::set_error("lsrtm_ex: NULL argument");
    if (niter < 0) return sepx::set_error("lsrtm_ex: niter %d < 0", niter);
    if (opts->policy != SEPX_DIR_FALLBACK && opts->policy != SEPX_DIR_ADAPTIVE)
      return sepx::set_error("lsrtm_ex: unknown direction policy %d", opts->policy);
    auto *b = static_cast<op_box *>(h);
    b->data->upload(data);
    cgstep st;
    simple_solver solv(&st, b->data.get(), b->op.get());
    solv.dir = opts->dir;
    solv.dir_ctx = opts->dir_ctx;
    solv.dir_policy = opts->policy;
    solv.fallback_ratio = opts->fallback_ratio;
    solv.probe_every = opts->probe_every;
    solv.target = opts->target;
    solv.solve(niter);
    std::unique_ptr<my_vector> mod(solv.return_model());
    hf(mod.get())->download(model);
    const size_t done = solv.resid.size();
    for (size_t i = 0; i < (size_t)niter; i++) {
      const bool ran = i < done;
      if (resid) resid[i] = ran ? solv.resid[i] : -1.0;
      if (seconds) seconds[i] = ran ? solv.seconds[i] : -1.0;
      if (used_dir) used_dir[i] = ran ? solv.used_dir[i] : -1;
    }
    if (iters_done) *iters_done = (int)done;
    return 0;
  } catch (const std::exception &e) {
    return sepx::set_error("lsrtm_ex: %s", e.what());
  }
}

}  // extern "C"

// ------------------------------------------------------------------ tmute, image, data
namespace {
// first cell of a window in the grid of `out`, as image_rtm_3d computes it
// (Born/image_rtm_3d.cpp:33-35): (int)((o_in - o_out) / d_out) in float
int window_offset(const axis &in, const axis &out) { return (int)((in.o - out.o) / out.d); }

void need3(const hypercube_float *h, const char *what) {
  if (h->axes.size() < 3) throw std::runtime_error(std::string(what) + ": needs three axes");
}
}  // namespace

tmute::tmute(float t, float v, my_vector *mod, my_vector *dat) : t_0(t), vmute(v) {
  set_domain(mod);
  set_range(dat);
}

static void tmute_apply(bool adj, bool add, float t0, float vm, my_vector *model, my_vector *data) {
  auto *m = hf(model), *d = hf(data);
  if (m->n123 != d->n123 || d->axes.size() < 2) throw std::runtime_error("tmute: shapes differ");
  const axis a1 = d->get_axis(1), a2 = d->get_axis(2);
  const long long nrep = d->n123 / ((long long)a1.n * a2.n);
  ck(sepx_tmute(adj ? 1 : 0, add ? 1 : 0, t0, vm, a1.n, a1.o, a1.d, a2.n, a2.o, a2.d, nrep, m->vals,
                d->vals),
     "tmute");
}

bool tmute::forward(bool add, my_vector *model, my_vector *data, int) {
  tmute_apply(false, add, t_0, vmute, model, data);
  return true;
}

bool tmute::adjoint(bool add, my_vector *model, my_vector *data, int) {
  tmute_apply(true, add, t_0, vmute, model, data);
  return true;
}

image_rtm_3d::image_rtm_3d(const std::vector<axis> &axes) {
  if (axes.size() != 3) throw std::runtime_error("image_rtm_3d: needs three axes");
  image = new hypercube_float(axes);
}

image_rtm_3d::image_rtm_3d(const char *, const vel_fd_3d *vel) {
  if (!vel || vel->axes.size() != 3) throw std::runtime_error("image_rtm_3d: needs a 3-D velocity");
  image = new hypercube_float(vel->axes);
  image->zero();
}

// ------------------------------------------------------------------ inputs of the
// reference's rtm_zero_op constructor
int param_func::get_int(const char *arg, int def) const {
  auto it = vals.find(arg ? arg : "");
  return it == vals.end() ? def : (int)it->second;
}

float param_func::get_float(const char *arg, float def) const {
  auto it = vals.find(arg ? arg : "");
  return it == vals.end() ? def : (float)it->second;
}

param_func &param_func::set(const std::string &name, double value) {
  vals[name] = value;
  return *this;
}

vel_fd_3d::vel_fd_3d(const std::vector<axis> &ax, const float *vel) : axes(ax) {
  if (ax.size() != 3 || !vel) throw std::runtime_error("vel_fd_3d: needs three axes and values");
  vals.assign(vel, vel + (size_t)ax[0].n * ax[1].n * ax[2].n);
}

float vel_fd_3d::max_vel() const {
  float m = vals.empty() ? 0.f : vals[0];
  for (float v : vals) m = std::max(m, v);
  return m;
}

float vel_fd_3d::min_vel() const {
  float m = vals.empty() ? 0.f : vals[0];
  for (float v : vals) m = std::min(m, v);
  return m;
}

float vel_fd_3d::get_min_samp() const {
  const float dx = axes[0].d, dy = axes[1].d, dz = axes[2].d;
  if (dz < dx && dz < dy) return dz;
  if (dy < dx) return dz;
  return dx;
}

float vel_fd_3d::get_max_samp() const {
  const float dx = axes[0].d, dy = axes[1].d, dz = axes[2].d;
  if (dz > dx && dz > dy) return dz;
  if (dy > dx) return dz;
  return dx;
}

source_func::source_func(axis t, const float *w) : at(t) {
  if (!w || t.n < 1) throw std::runtime_error("source_func: empty wavelet");
  wavelet.assign(w, w + t.n);
}

void source_func::set_sources_3d(float s_z, axis a_sx, axis a_sy) {
  for (int i2 = 0; i2 < a_sy.n; i2++)
    for (int i1 = 0; i1 < a_sx.n; i1++) {
      sz.push_back(s_z);
      sx.push_back(a_sx.o + a_sx.d * i1);
      sy.push_back(a_sy.o + a_sy.d * i2);
    }
}

image_rtm_3d::~image_rtm_3d() {
  delete image;
  delete mute;
}

void image_rtm_3d::set_mute(const hypercube_float &m) {
  if (m.n123 != image->n123) throw std::runtime_error("image_rtm_3d: mute shape differs");
  if (!mute) mute = new hypercube_float(image->axes);
  ck(sepx_vec_copy(mute->vals, m.vals, m.n123), "set_mute");
}

void image_rtm_3d::add_image(const hypercube_float *img) {
  need3(img, "add_image");
  const axis o1 = get_axis(1), o2 = get_axis(2), o3 = get_axis(3);
  const axis i1 = img->get_axis(1), i2 = img->get_axis(2), i3 = img->get_axis(3);
  ck(sepx_image_add_window(image->vals, o1.n, o2.n, o3.n, window_offset(i1, o1),
                           window_offset(i2, o2), window_offset(i3, o3), img->vals, i1.n, i2.n,
                           i3.n),
     "add_image");
}

hypercube_float *image_rtm_3d::extract_sub(axis a1, axis a2, axis a3) const {
  const axis o1 = get_axis(1), o2 = get_axis(2), o3 = get_axis(3);
  std::unique_ptr<hypercube_float> sub(new hypercube_float({a1, a2, a3}));
  ck(sepx_image_extract_window(image->vals, mute ? mute->vals : nullptr, o1.n, o2.n, o3.n,
                               window_offset(a1, o1), window_offset(a2, o2), window_offset(a3, o3),
                               sub->vals, a1.n, a2.n, a3.n),
     "extract_sub");
  return sub.release();
}

void image_rtm_3d::write_volume() {
  if (mute) image->mult(mute);
}

data_rtm_3d::data_rtm_3d(const std::vector<axis> &ax) : hypercube_float(ax) {
  if (ax.size() < 3) throw std::runtime_error("data_rtm_3d: needs (t, x, y[, shots]) axes");
}

data_rtm_3d::data_rtm_3d(const std::vector<axis> &ax, const param_func *par) : data_rtm_3d(ax) {
  sz = par ? par->get_float("rec_depth", 0.f) : 0.f;
}

int data_rtm_3d::nshots() const {
  int n = 1;
  for (size_t i = 3; i < axes.size(); i++) n *= axes[i].n;
  return n;
}

void data_rtm_3d::add_data(int ishot, const hypercube_float *dat) {
  const long long slab = (long long)axes[0].n * axes[1].n * axes[2].n;
  if (ishot < 0 || ishot >= nshots()) throw std::runtime_error("add_data: shot out of range");
  if (dat->n123 != slab) throw std::runtime_error("add_data: the shot's size differs");
  ck(sepx_vec_add(vals + (long long)ishot * slab, dat->vals, slab), "add_data");
}
