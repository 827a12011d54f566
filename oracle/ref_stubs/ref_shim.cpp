// C entry points into the reference's own host C++ (compiled from its sources
// by oracle/build_oracle.py), so that tests can compare the oracle and the
// product against the reference code itself.  Test infrastructure only.
#include <cstdio>
#include <cstring>
#include <vector>

#include "cgstep.h"
#include "deriv_3d.h"
#include "float_3d.h"
#include "data_rtm_3d.h"
#include "hypercube_float.h"
#include "image_rtm_3d.h"
#include "laplac_3d.h"
#include "lin_solver.h"
#include "map_data_3d.h"
#include "sinc_bob.h"
#include "source_func_3d.h"
#include "tmute.h"
#include "vel_fd_3d.h"

namespace {
std::vector<axis> axes3(int n1, float o1, float d1, int n2, float o2, float d2, int n3, float o3,
                        float d3) {
  std::vector<axis> a;
  a.push_back(axis(n1, o1, d1));
  a.push_back(axis(n2, o2, d2));
  a.push_back(axis(n3, o3, d3));
  return a;
}

// float_3d whose storage has one spare element: deriv_3d.cpp reads and writes
// one sample past the last trace.
float_3d *padded_cube(int n1, int n2, int n3, const float *init, float d1 = 1.f) {
  float_3d *c = new float_3d(axis(n1, 0.f, d1), axis(n2), axis(n3));
  long n = (long)n1 * n2 * n3;
  delete[] c->vals;
  c->vals = new float[n + 1];
  if (init) memcpy(c->vals, init, sizeof(float) * n);
  else memset(c->vals, 0, sizeof(float) * n);
  c->vals[n] = 0.f;
  return c;
}

// Dense matrix operator used to drive the reference solver on small problems.
class dense_op : public my_operator {
 public:
  dense_op(const float *a, int nr, int nc, hypercube_float *dom, hypercube_float *ran)
      : A(a), nr(nr), nc(nc) {
    set_domain(dom);
    set_range(ran);
  }
  virtual bool forward(bool add, my_vector *model, my_vector *data, int iter = 1) {
    hypercube_float *m = (hypercube_float *)model, *d = (hypercube_float *)data;
    if (!add) d->zero();
    for (int i = 0; i < nr; i++) {
      double s = 0;
      for (int j = 0; j < nc; j++) s += (double)A[(long)i * nc + j] * m->vals[j];
      d->vals[i] += (float)s;
    }
    return true;
  }
  virtual bool adjoint(bool add, my_vector *model, my_vector *data, int iter = 1) {
    hypercube_float *m = (hypercube_float *)model, *d = (hypercube_float *)data;
    if (!add) m->zero();
    for (int j = 0; j < nc; j++) {
      double s = 0;
      for (int i = 0; i < nr; i++) s += (double)A[(long)i * nc + j] * d->vals[i];
      m->vals[j] += (float)s;
    }
    return true;
  }
  const float *A;
  int nr, nc;
};
}  // namespace

extern "C" {

void ref_sinc_table(int ntab, int nsinc, float *out) {
  sinc_bob s(ntab, nsinc);
  for (int it = 0; it < ntab; it++) memcpy(out + (long)it * nsinc, s.table[it], sizeof(float) * nsinc);
}

void ref_rand_subspace(int irand, int nrand1, int nrand2, int nrand3, float dt, const float *model,
                       int m1, int m2, int m3, float mo1, float mo2, float mo3, float md1, float md2,
                       float md3, int s1, int s2, int s3, float so1, float so2, float so3, float sd1,
                       float sd2, float sd3, float *out) {
  vel_fd_3d v;
  v.fld = new hypercube_float(axes3(m1, mo1, md1, m2, mo2, md2, m3, mo3, md3));
  memcpy(v.fld->vals, model, sizeof(float) * (long)m1 * m2 * m3);
  hypercube_float space(axes3(s1, so1, sd1, s2, so2, sd2, s3, so3, sd3), false);
  hypercube_float *r = v.rand_subspace(irand, nrand1, nrand2, nrand3, dt, &space);
  memcpy(out, r->vals, sizeof(float) * (long)s1 * s2 * s3);
  delete r;
}

// source_func::set_compute_size + create_domain: padded sizes and origins
void ref_compute_domain(int m1, int m2, int m3, float md1, float md2, float md3, int nbt, int nb,
                        int nby, int fat, int n[3], float o[3]) {
  source_func sf;
  sf.wavelet = 0;
  hypercube dom;
  dom.set_axes(axes3(m1, 0.f, md1, m2, 0.f, md2, m3, 0.f, md3));
  sf.set_compute_size(&dom, 8.f, nbt, nb, nby, fat, 16);
  hypercube_float *d = sf.create_domain(0);
  for (int k = 0; k < 3; k++) {
    n[k] = d->get_axis(k + 1).n;
    o[k] = d->get_axis(k + 1).o;
  }
  delete d;
}

void ref_file_put(const char *tag, int ndim, const int *n, const float *o, const float *d,
                  const void *data, long nbytes);

// source_func constructor (wavelet time derivative) reading an in-memory file
void ref_wavelet_deriv(const float *w, int n, float o, float d, float *out) {
  int nn = n;
  float oo = o, dd = d;
  ref_file_put("wavelet", 1, &nn, &oo, &dd, w, (long)n * 4);
  source_func sf((char *)"wavelet");
  memcpy(out, sf.wavelet->vals, sizeof(float) * n);
}

// source_func::get_source_func with a given (already differentiated) wavelet
void ref_source_func(const float *wav, int nwav, float dtw, float sx, float sy, float sz, int n1,
                     int n2, int n3, float o1, float o2, float o3, float d1, float d2, float d3,
                     int nts, int *locs, float *vals) {
  source_func sf;
  std::vector<axis> wa;
  wa.push_back(axis(nwav, 0.f, dtw));
  sf.set_axes(wa);
  sf.wavelet = new hypercube_float(wa);
  memcpy(sf.wavelet->vals, wav, sizeof(float) * nwav);
  sf.sx.push_back(sx);
  sf.sy.push_back(sy);
  sf.sz.push_back(sz);
  hypercube_float dom(axes3(n1, o1, d1, n2, o2, d2, n3, o3, d3), false);
  sf.get_source_func(&dom, 0, nts, locs, vals);
}

void ref_deriv(int fwd, int add, int nt, int n2, int n3, float dt, float *m, float *d) {
  float_3d *mm = padded_cube(nt, n2, n3, m, dt), *dd = padded_cube(nt, n2, n3, d, dt);
  deriv op(mm, dd);
  if (fwd) op.forward(add != 0, mm, dd);
  else op.adjoint(add != 0, mm, dd);
  long n = (long)nt * n2 * n3;
  memcpy(m, mm->vals, sizeof(float) * n);
  memcpy(d, dd->vals, sizeof(float) * n);
  delete mm;
  delete dd;
}

void ref_laplac(int fwd, int add, int n1, int n2, int n3, float *m, float *d) {
  float_3d *mm = padded_cube(n1, n2, n3, m), *dd = padded_cube(n1, n2, n3, d);
  laplac op(mm, dd);
  if (fwd) op.forward(add != 0, mm, dd);
  else op.adjoint(add != 0, mm, dd);
  long n = (long)n1 * n2 * n3;
  memcpy(m, mm->vals, sizeof(float) * n);
  memcpy(d, dd->vals, sizeof(float) * n);
  delete mm;
  delete dd;
}

void ref_map_data(int fwd, int add, int ntb, int nt, int n2, int n3, float *m, float *d) {
  float_3d *mm = padded_cube(ntb, n2, n3, m), *dd = padded_cube(nt, n2, n3, d);
  int npt = n2 * n3;
  std::vector<float> sx(npt, 0.f), sy(npt, 0.f), sz(npt, 0.f);
  std::vector<int> locs(npt, 0);
  float_3d model(4, 4, 4);
  map_data op(npt, sx.data(), sy.data(), sz.data(), locs.data(), &model, mm, dd, ntb);
  if (fwd) op.forward(add != 0, mm, dd);
  else op.adjoint(add != 0, mm, dd);
  memcpy(m, mm->vals, sizeof(float) * (long)ntb * n2 * n3);
  memcpy(d, dd->vals, sizeof(float) * (long)nt * n2 * n3);
  delete mm;
  delete dd;
}

// simple_solver + cgstep (Born/lin_solver.cpp, Born/cgstep.cpp) on a dense
// least-squares problem A m = d; returns the model and the residual energy.
int ref_cg_solve(const float *A, int nr, int nc, const float *d, int niter, float *m_out,
                 double *rr_out) {
  std::vector<axis> ma, da;
  ma.push_back(axis(nc));
  da.push_back(axis(nr));
  hypercube_float mod(ma), dat(da);
  mod.zero();
  memcpy(dat.vals, d, sizeof(float) * nr);
  dense_op op(A, nr, nc, &mod, &dat);
  cgstep *st = new cgstep();
  simple_solver *solv = new simple_solver(st, &dat, &op);
  bool ok = solv->solve(niter);
  hypercube_float *m = (hypercube_float *)solv->return_model();
  memcpy(m_out, m->vals, sizeof(float) * nc);
  *rr_out = solv->rr->dot(solv->rr);
  delete m;
  return ok ? 0 : 1;
}

// my_operator::dot_test on the dense operator (tolerance 1e-4, Born/my_operator.cpp:14-76)
int ref_dense_dot_test(const float *A, int nr, int nc, unsigned int seed) {
  std::vector<axis> ma, da;
  ma.push_back(axis(nc));
  da.push_back(axis(nr));
  hypercube_float mod(ma), dat(da);
  dense_op op(A, nr, nc, &mod, &dat);
  srand(seed);
  return op.dot_test(false) ? 1 : 0;
}

void ref_file_put(const char *tag, int ndim, const int *n, const float *o, const float *d,
                  const void *data, long nbytes);
long ref_file_get(const char *tag, void *out, long nbytes);

// ---- image / data vectors (Born/image_rtm_3d.cpp, data_rtm_3d.cpp, tmute.cpp) ----

// image_rtm_3d over a grid (n, o, d): the constructor takes the axes of the
// velocity model it is given
static image_rtm_3d *make_image(const int n[3], const float o[3], const float d[3]) {
  vel_fd_3d *v = new vel_fd_3d();
  v->fld = new hypercube_float(axes3(n[0], o[0], d[0], n[1], o[1], d[1], n[2], o[2], d[2]));
  image_rtm_3d *im = new image_rtm_3d((char *)"ref_image", v);
  delete v;   // deletes fld
  return im;
}

// image_rtm_3d::add_image: img (in/out) on grid (n, o, d), sub on (sn, so, sd)
void ref_image_add(const int n[3], const float o[3], const float d[3], float *img, const int sn[3],
                   const float so[3], const float sd[3], const float *sub) {
  image_rtm_3d *im = make_image(n, o, d);
  const long nn = (long)n[0] * n[1] * n[2], ns = (long)sn[0] * sn[1] * sn[2];
  memcpy(im->image->vals, img, sizeof(float) * nn);
  hypercube_float s(axes3(sn[0], so[0], sd[0], sn[1], so[1], sd[1], sn[2], so[2], sd[2]));
  memcpy(s.vals, sub, sizeof(float) * ns);
  im->add_image(&s);
  memcpy(img, im->image->vals, sizeof(float) * nn);
  delete im;
}

// image_rtm_3d::extract_sub with the image read from its dataset and the
// "mute" dataset; also returns write_volume's muted image (image * mute)
void ref_image_extract(const int n[3], const float o[3], const float d[3], const float *img,
                       const float *mute, const int sn[3], const float so[3], const float sd[3],
                       float *sub, float *muted) {
  const long nn = (long)n[0] * n[1] * n[2], ns = (long)sn[0] * sn[1] * sn[2];
  ref_file_put("ref_image_src", 3, n, o, d, img, nn * 4);
  ref_file_put("mute", 3, n, o, d, mute, nn * 4);
  image_rtm_3d *im = make_image(n, o, d);
  oc_float src((char *)"ref_image_src");
  im->set_source_file(&src);
  float_3d *r = im->extract_sub(axis(sn[0], so[0], sd[0]), axis(sn[1], so[1], sd[1]),
                                axis(sn[2], so[2], sd[2]));
  memcpy(sub, r->vals, sizeof(float) * ns);
  delete r;
  // write_volume multiplies the image it holds by the mute once more
  ref_file_put("ref_image_src", 3, n, o, d, img, nn * 4);
  im->set_source_file(&src);
  im->write_volume();
  memcpy(muted, im->image->vals, sizeof(float) * nn);
  delete im;
}

// data_rtm_3d::add_data into a dataset of axes (n1, n2, n3, nshots)
void ref_add_data(int n1, int n2, int n3, int nshots, float *all, int ishot, const float *shot) {
  const int n[4] = {n1, n2, n3, nshots};
  const float o[4] = {0.f, 0.f, 0.f, 0.f}, d[4] = {1.f, 1.f, 1.f, 1.f};
  const long slab = (long)n1 * n2 * n3;
  ref_file_put("ref_data", 4, n, o, d, all, slab * nshots * 4);
  data_rtm_3d dat;
  dat.init_nd(std::vector<axis>{axis(n1), axis(n2), axis(n3), axis(nshots)});
  oc_float f((char *)"ref_data");
  dat.set_source_file(&f);
  hypercube_float h(axes3(n1, 0.f, 1.f, n2, 0.f, 1.f, n3, 0.f, 1.f));
  memcpy(h.vals, shot, sizeof(float) * slab);
  dat.add_data(ishot, &h);
  ref_file_get("ref_data", all, slab * nshots * 4);
}

// tmute::forward / adjoint on datasets of axes (t, x, n3, n4, n5)
void ref_tmute(int fwd, int add, float t0, float vmute, int n1, float o1, float d1, int n2, float o2,
               float d2, int n3, int n4, int n5, float *model, float *data) {
  const int n[5] = {n1, n2, n3, n4, n5};
  const float o[5] = {o1, o2, 0.f, 0.f, 0.f}, d[5] = {d1, d2, 1.f, 1.f, 1.f};
  const long nb = (long)n1 * n2 * n3 * n4 * n5 * 4;
  ref_file_put("ref_tm_model", 5, n, o, d, model, nb);
  ref_file_put("ref_tm_data", 5, n, o, d, data, nb);
  oc_float m((char *)"ref_tm_model"), dd((char *)"ref_tm_data");
  tmute op(t0, vmute, &m, &dd);
  if (fwd) op.forward(add != 0, &m, &dd);
  else op.adjoint(add != 0, &m, &dd);
  ref_file_get("ref_tm_model", model, nb);
  ref_file_get("ref_tm_data", data, nb);
}

}  // extern "C"
