// The solver layer of the operator API on the GPU (tests/test_gpu_solvers.py
// builds and runs it): simple_solver + cgstep, prec_solver, reg_solver,
// row_op and col_op on dense test operators over device vectors.  The dense
// operator does what the reference harness's dense_op does (each output an
// FP64 sum in index order, rounded to float, added in float), on the host;
// every vector operation of the solvers runs on the device.
//
//   <dir>/dims.bin: nr nc nq nb nc2 K K2 eps  (float32)
//   A [nr][nc], P [nc][nc], R [nq][nc], B [nb][nr], C [nc2][nc], d [nr],
//   x [nc], yb [nb], yr [nr], yc [nc2]        -> results beside them
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "sepx.h"
#include "sepx_ops.h"

static std::string g_dir;

static std::vector<float> load(const char *name, size_t n) {
  std::vector<float> v(n);
  FILE *f = fopen((g_dir + "/" + name + ".bin").c_str(), "rb");
  if (!f || fread(v.data(), sizeof(float), n, f) != n) throw std::runtime_error(name);
  fclose(f);
  return v;
}

static void save(const std::string &name, const void *p, size_t bytes) {
  FILE *f = fopen((g_dir + "/" + name + ".bin").c_str(), "wb");
  if (!f || fwrite(p, 1, bytes, f) != bytes) throw std::runtime_error(name);
  fclose(f);
}

static hypercube_float *hc(my_vector *v) {
  auto *h = dynamic_cast<hypercube_float *>(v);
  if (!h) throw std::runtime_error("expected a hypercube_float");
  return h;
}

static std::vector<float> host(my_vector *v) {
  hypercube_float *h = hc(v);
  std::vector<float> out((size_t)h->n123);
  h->download(out.data());
  return out;
}

static void save_vec(const std::string &name, my_vector *v) {
  std::vector<float> out;
  if (auto *s = dynamic_cast<super_vector *>(v)) {
    for (my_vector *p : s->vecs) {
      std::vector<float> part = host(p);
      out.insert(out.end(), part.begin(), part.end());
    }
  } else {
    out = host(v);
  }
  save(name, out.data(), out.size() * sizeof(float));
}

// y (+)= scale * A x, A dense [nr][nc] in host memory
class dense_op : public my_operator {
 public:
  dense_op(const std::vector<float> &a, int nr_, int nc_) : A(a), nr(nr_), nc(nc_) {
    hypercube_float dom({axis(nc)}), ran({axis(nr)});
    set_domain(&dom);
    set_range(&ran);
  }
  bool forward(bool add, my_vector *model, my_vector *data, int) override {
    std::vector<float> m = host(model), d((size_t)nr, 0.f);
    if (add) d = host(data);
    for (int i = 0; i < nr; i++) {
      double s = 0;
      for (int j = 0; j < nc; j++) s += (double)A[(size_t)i * nc + j] * m[j];
      d[i] += (float)(scale == 1.f ? s : s * (double)scale);
    }
    hc(data)->upload(d.data());
    return true;
  }
  bool adjoint(bool add, my_vector *model, my_vector *data, int) override {
    std::vector<float> d = host(data), m((size_t)nc, 0.f);
    if (add) m = host(model);
    for (int j = 0; j < nc; j++) {
      double s = 0;
      for (int i = 0; i < nr; i++) s += (double)A[(size_t)i * nc + j] * d[i];
      m[j] += (float)(scale == 1.f ? s : s * (double)scale);
    }
    hc(model)->upload(m.data());
    return true;
  }
  std::vector<float> A;
  int nr, nc;
};

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  g_dir = argv[1];
  try {
    if (sepx_setup_cuda(1)) throw std::runtime_error(sepx_last_error());
    const std::vector<float> D = load("dims", 8);
    const int nr = (int)D[0], nc = (int)D[1], nq = (int)D[2], nb = (int)D[3], nc2 = (int)D[4];
    const int K = (int)D[5], K2 = (int)D[6];
    const float eps = D[7];
    dense_op A(load("A", (size_t)nr * nc), nr, nc);
    dense_op P(load("P", (size_t)nc * nc), nc, nc);
    dense_op R(load("R", (size_t)nq * nc), nq, nc);
    dense_op B(load("B", (size_t)nb * nr), nb, nr);
    dense_op Cm(load("C", (size_t)nc2 * nc), nc2, nc);
    hypercube_float data({axis(nr)});
    data.upload(load("d", nr).data());

    // simple_solver + cgstep: the model after k = 1 .. K iterations, each from
    // m = 0, and rr.rr of the K-iteration run
    std::vector<float> models;
    std::vector<double> resid;
    for (int k = 1; k <= K; k++) {
      cgstep st;
      simple_solver solv(&st, &data, &A);
      if (!solv.solve(k)) throw std::runtime_error("simple_solver stopped early");
      std::unique_ptr<my_vector> m(solv.return_model());
      std::vector<float> mh = host(m.get());
      models.insert(models.end(), mh.begin(), mh.end());
      if (k == K) resid = solv.resid;
    }
    save("simple_models", models.data(), models.size() * sizeof(float));
    save("simple_resid", resid.data(), resid.size() * sizeof(double));

    {  // [A P; eps I] x, model P x
      cgstep st;
      prec_solver solv(&st, &data, &A, &P, eps);
      solv.solve(K2);
      std::unique_ptr<my_vector> m(solv.return_model());
      save_vec("prec_model", m.get());
      save("prec_resid", solv.resid.data(), solv.resid.size() * sizeof(double));
    }
    {  // [A; eps I]
      hypercube_float dom({axis(nc)});
      i_op I(&dom, &dom);
      cgstep st;
      reg_solver solv(&st, &data, &A, &I, eps);
      solv.solve(K2);
      std::unique_ptr<my_vector> m(solv.return_model());
      save_vec("reg_i_model", m.get());
      save("reg_i_resid", solv.resid.data(), solv.resid.size() * sizeof(double));
    }
    {  // [A; eps R]
      cgstep st;
      reg_solver solv(&st, &data, &A, &R, eps);
      solv.solve(K2);
      std::unique_ptr<my_vector> m(solv.return_model());
      save_vec("reg_r_model", m.get());
      save("reg_r_resid", solv.resid.data(), solv.resid.size() * sizeof(double));
      R.set_scale(1.f);
    }
    // row_op: B A;  col_op: [A; C]
    hypercube_float x({axis(nc)});
    x.upload(load("x", nc).data());
    {
      row_op op({&A, &B});
      std::unique_ptr<my_vector> y(op.range->clone_zero()), xa(op.domain->clone_zero());
      op.forward(false, &x, y.get());
      save_vec("row_fwd", y.get());
      std::unique_ptr<my_vector> yb(op.range->clone_zero());
      hc(yb.get())->upload(load("yb", nb).data());
      op.adjoint(false, xa.get(), yb.get());
      save_vec("row_adj", xa.get());
      double dots[4];
      op.dot_test(false, dots);
      save("row_dot", dots, sizeof dots);
    }
    {
      col_op op({&A, &Cm});
      std::unique_ptr<my_vector> y(op.range->clone_zero()), xa(op.domain->clone_zero());
      op.forward(false, &x, y.get());
      save_vec("col_fwd", y.get());
      std::unique_ptr<my_vector> yy(op.range->clone_zero());
      auto *sv = dynamic_cast<super_vector *>(yy.get());
      hc(sv->vecs[0])->upload(load("yr", nr).data());
      hc(sv->vecs[1])->upload(load("yc", nc2).data());
      op.adjoint(false, xa.get(), yy.get());
      save_vec("col_adj", xa.get());
      double dots[4];
      op.dot_test(false, dots);
      save("col_dot", dots, sizeof dots);
    }
  } catch (const std::exception &e) {
    fprintf(stderr, "solver_driver: %s\n", e.what());
    return 1;
  }
  return 0;
}
