/*
 * sepx_ops.h -- the operator / vector / solver layer of SEP_Code's Born path
 * on device-resident vectors: the reference's classes and methods
 * (Born/my_vector.h, hypercube_float.h, super_vector.h, my_operator.h,
 * combo_oper.h, i_op.h, step.h, cgstep.h, lin_solver.h, rtm_zero_op_3d.h)
 * with the same names and semantics -- `add` accumulates, dot products and
 * step lengths in FP64 -- over the C ABI of include/sepx.h.  SEPlib-file
 * arguments are replaced by in-memory descriptions (rtm_problem).
 *
 * Part 2 (extern "C") exposes the operator and the least-squares solver to
 * callers without C++ (Python tests and benchmarks use it through ctypes).
 */
#ifndef SEPX_OPS_H
#define SEPX_OPS_H

#ifdef __cplusplus
extern "C" {
#endif

/* One survey: what the reference reads from its SEP files for rtm_zero_op. */
typedef struct {
  const float *vel;          /* model velocity, host float[m3][m2][m1] (m/s) */
  int m1, m2, m3;
  float d1, d2, d3;          /* grid spacing (origins: mo1..mo3 below) */
  const float *wavelet;      /* source wavelet before its time derivative */
  int nwav;
  float dtw;
  int data_nt;               /* samples per recorded trace */
  float data_dt;
  int rnx, rny;              /* receiver grid (data axes 2, 3) */
  float ro2, rd2, ro3, rd3;
  float rec_depth;
  int nshots;
  const float *shot_xyz;     /* host float[nshots][3] (x, y, z) */
  int nbound;                /* random boundary / sponge width (cells) */
  float bc_a, bc_b;          /* sponge */
  int mode;                  /* 0: the reference's rtm_forward / rtm_adjoint
                                1: the exact-adjoint linearised pair */
  int snap_js;               /* mode 1: snapshot interval (steps) */
  int snap_prec;             /* mode 1: 0 FP32, 1 BF16, 2 FP16 */
  float mo1, mo2, mo3;       /* origins of the velocity / image grid (0 if unset) */
} sepx_rtm_problem;

typedef void *sepx_op_handle;

/* preconditioner of the search direction: g <- P(g) on device memory */
typedef int (*sepx_direction_fn)(void *ctx, float *g, long long n);

sepx_op_handle sepx_rtm_op_create(const sepx_rtm_problem *p);
void sepx_rtm_op_destroy(sepx_op_handle op);
/* element counts of the operator's model and data vectors (-1: NULL op) */
long long sepx_rtm_op_model_size(sepx_op_handle op);
long long sepx_rtm_op_data_size(sepx_op_handle op);
/* host-buffer forward / adjoint (rtm_zero_op::forward / ::adjoint) */
int sepx_rtm_op_forward(sepx_op_handle op, int add, const float *model, float *data);
int sepx_rtm_op_adjoint(sepx_op_handle op, int add, float *model, const float *data);
/* my_operator::dot_test: out = {<L m1, d2>, <m2, L' d2>, add=true pair} */
int sepx_rtm_op_dot_test(sepx_op_handle op, unsigned long long seed, double out[4]);
/* least-squares RTM with simple_solver + cgstep (Born/lin_solver.cpp:7,
 * :115-143; Born/cgstep.cpp:14-58): niter iterations from m = 0; writes the
 * model, the FP64 residual energy rr.rr after each iteration and the wall
 * seconds at each iteration; `dir` (may be NULL) preconditions the search
 * direction g before the forward product.  fallback_ratio > 0: once a
 * preconditioned iteration leaves rr.rr above fallback_ratio times its
 * previous value, the remaining iterations use plain g (the iteration is
 * written to *fallback_iter, -1 if none; may be NULL). */
int sepx_lsrtm(sepx_op_handle op, const float *data, int niter, float *model, double *resid,
               double *seconds, sepx_direction_fn dir, void *dir_ctx, double fallback_ratio,
               int *fallback_iter);

/* When the search direction is preconditioned (the learned direction of the
 * least-squares RTM; no counterpart in the reference, whose solver is plain
 * Born/lin_solver.cpp:115-143):
 *  SEPX_DIR_FALLBACK  as sepx_lsrtm: preconditioned until one step lowers
 *                     rr.rr by less than fallback_ratio allows, then plain g;
 *  SEPX_DIR_ADAPTIVE  preconditioned while its steps lower rr.rr by at least
 *                     as large a fraction as the latest plain step did (before
 *                     the first plain step: the fallback_ratio rule); after a
 *                     switch to plain g the preconditioned direction is tried
 *                     again every probe_every plain iterations. */
enum { SEPX_DIR_FALLBACK = 0, SEPX_DIR_ADAPTIVE = 1 };
typedef struct {
  sepx_direction_fn dir;   /* NULL: plain simple_solver + cgstep */
  void *dir_ctx;
  int policy;              /* SEPX_DIR_FALLBACK | SEPX_DIR_ADAPTIVE */
  double fallback_ratio;
  int probe_every;         /* SEPX_DIR_ADAPTIVE, >= 1 */
  double target;           /* > 0: stop once sqrt(rr.rr / rr0.rr0) <= target */
} sepx_lsrtm_opts;
/* sepx_lsrtm with a direction policy and a stopping residual: runs at most
 * niter iterations; resid / seconds / used_dir (1 where the preconditioned
 * direction was used; each may be NULL) are written for the iterations run,
 * -1 after them; *iters_done (may be NULL) is the number run. */
int sepx_lsrtm_ex(sepx_op_handle op, const float *data, int niter, const sepx_lsrtm_opts *opts,
                  float *model, double *resid, double *seconds, int *used_dir, int *iters_done);

#ifdef __cplusplus
}

#include <map>
#include <string>
#include <vector>

struct axis {
  int n = 1;
  float o = 0.f, d = 1.f;
  axis() {}
  axis(int n_, float o_ = 0.f, float d_ = 1.f) : n(n_), o(o_), d(d_) {}
};

// Abstract vector (Born/my_vector.h:10-48).
class my_vector {
 public:
  virtual ~my_vector() {}
  virtual my_vector *clone_vec() = 0;     // copy
  virtual my_vector *clone_space() = 0;   // same space, zero-filled
  virtual my_vector *clone_zero();
  virtual void scale(double num) = 0;
  virtual void scale_add(double mes, my_vector *vec, double other) = 0;   // this = this*mes + vec*other
  virtual void scale_add(double sc1, my_vector *v1, double sc2, my_vector *v2) = 0;   // v1*sc1 + v2*sc2
  virtual void set_val(double val) = 0;
  virtual void add(my_vector *vec) = 0;
  virtual void mult(my_vector *vec) = 0;
  virtual double sum() = 0;
  virtual double dot(my_vector *vec) = 0;   // FP64 accumulation
  virtual void random() = 0;                // uniform(-0.5, 0.5)
  virtual bool check_match(const my_vector *v2) const = 0;
  void zero() { set_val(0.); }
  std::string name;
};

// Device-resident float hypercube (Born/hypercube_float.h).
class hypercube_float : public my_vector {
 public:
  explicit hypercube_float(const std::vector<axis> &axes);
  hypercube_float(const hypercube_float &) = delete;
  ~hypercube_float() override;
  my_vector *clone_vec() override;
  my_vector *clone_space() override;
  void scale(double num) override;
  void scale_add(double mes, my_vector *vec, double other) override;
  void scale_add(double sc1, my_vector *v1, double sc2, my_vector *v2) override;
  void set_val(double val) override;
  void add(my_vector *vec) override;
  void mult(my_vector *vec) override;
  double sum() override;
  double dot(my_vector *vec) override;
  void random() override;
  bool check_match(const my_vector *v2) const override;
  void upload(const float *host);
  void download(float *host) const;
  long long get_n123() const { return n123; }
  axis get_axis(int i) const { return axes[i - 1]; }
  std::vector<axis> axes;
  long long n123 = 0;
  float *vals = nullptr;   // device memory
};

// Concatenation of vectors (Born/super_vector.h).
class super_vector : public my_vector {
 public:
  explicit super_vector(const std::vector<my_vector *> &vs, bool just_space = false);
  ~super_vector() override;
  my_vector *clone_vec() override;
  my_vector *clone_space() override;
  void scale(double num) override;
  void scale_add(double mes, my_vector *vec, double other) override;
  void scale_add(double sc1, my_vector *v1, double sc2, my_vector *v2) override;
  void set_val(double val) override;
  void add(my_vector *vec) override;
  void mult(my_vector *vec) override;
  double sum() override;
  double dot(my_vector *vec) override;
  void random() override;
  bool check_match(const my_vector *v2) const override;
  std::vector<my_vector *> vecs;
};

// Abstract linear operator (Born/my_operator.h:5-35).
class my_operator {
 public:
  virtual ~my_operator();
  virtual bool forward(bool add, my_vector *model, my_vector *data, int iter = 1) = 0;
  virtual bool adjoint(bool add, my_vector *model, my_vector *data, int iter = 1) = 0;
  void set_domain(my_vector *dom);
  void set_range(my_vector *ran);
  virtual void hessian(my_vector *in, my_vector *out);
  // random model / data, <L m1, d2> vs <m2, L' d2> with add false and true;
  // `out` (may be null) receives the four dot products
  bool dot_test(bool verb, double *out = nullptr, double tol = 1e-4);
  virtual void set_scale(float s) { scale = s; }
  float scale = 1.f;
  my_vector *domain = nullptr, *range = nullptr;
};

// scaled identity (Born/i_op.cpp)
class i_op : public my_operator {
 public:
  i_op(my_vector *mod, my_vector *dat);
  bool forward(bool add, my_vector *model, my_vector *data, int iter = 1) override;
  bool adjoint(bool add, my_vector *model, my_vector *data, int iter = 1) override;
};

// product op_n ... op_1 (Born/combo_oper.h: row_op)
class row_op : public my_operator {
 public:
  explicit row_op(const std::vector<my_operator *> &ops);
  ~row_op() override;
  bool forward(bool add, my_vector *model, my_vector *data, int iter = 1) override;
  bool adjoint(bool add, my_vector *model, my_vector *data, int iter = 1) override;
  std::vector<my_operator *> ops;
};

// stacked operators [op_1; op_2; ...] into a super_vector range (col_op)
class col_op : public my_operator {
 public:
  explicit col_op(const std::vector<my_operator *> &ops);
  bool forward(bool add, my_vector *model, my_vector *data, int iter = 1) override;
  bool adjoint(bool add, my_vector *model, my_vector *data, int iter = 1) override;
  std::vector<my_operator *> ops;
};

// Step rules (Born/step.h, Born/cgstep.h).
class step {
 public:
  virtual ~step() {}
  virtual void alloc_step(my_vector *mod, my_vector *dat) = 0;
  virtual bool step_it(int iter, my_vector *x, my_vector *g, my_vector *rr, my_vector *gg,
                       double *sc) = 0;
};

class cgstep : public step {
 public:
  ~cgstep() override;
  void alloc_step(my_vector *mod, my_vector *dat) override;
  bool step_it(int iter, my_vector *x, my_vector *g, my_vector *rr, my_vector *gg, double *sc) override;
  void forget_it();
  my_vector *s = nullptr, *ss = nullptr;
  bool forget = true;
  double small = 1e-20;
};

// Linear least-squares solvers (Born/lin_solver.h).
class lin_solver {
 public:
  virtual ~lin_solver();
  bool solve(int niter);
  virtual my_vector *return_model() { return m->clone_vec(); }
  void set_verbose(int v) { verb = v; }
  // optional preconditioning of the search direction before forward(g, gg)
  sepx_direction_fn dir = nullptr;
  void *dir_ctx = nullptr;
  double fallback_ratio = 0.0;   // > 0: switch to plain g once a step gains less
  int fallback_iter = -1;        // first iteration after which plain g was chosen
  int dir_policy = SEPX_DIR_FALLBACK;
  int probe_every = 8;
  double target = 0.0;           // > 0: stop at this residual relative to the initial one
  std::vector<double> resid, seconds;
  std::vector<int> used_dir;
  my_vector *g = nullptr, *m = nullptr, *gg = nullptr, *rr = nullptr;
  my_operator *oper = nullptr;
  step *st = nullptr;
  int verb = 0;

 protected:
  void init_solve(step *s);
  void create_solver_vecs();
  my_vector *init_rr(my_vector *data, my_operator *op, my_vector *m0);
  bool own_oper = false;
};

class simple_solver : public lin_solver {
 public:
  simple_solver(step *s, my_vector *data, my_operator *op, my_vector *m0 = nullptr);
};

// [L P; eps I] with model P x (Born/lin_solver.cpp:21-38)
class prec_solver : public lin_solver {
 public:
  prec_solver(step *s, my_vector *data, my_operator *op, my_operator *prec, float eps,
              my_vector *m0 = nullptr);
  ~prec_solver() override;
  my_vector *return_model() override;
  my_operator *pop = nullptr, *chain = nullptr, *iop = nullptr;
};

// [L; eps R] (Born/lin_solver.cpp:39-53)
class reg_solver : public lin_solver {
 public:
  reg_solver(step *s, my_vector *data, my_operator *op, my_operator *reg, float eps,
             my_vector *m0 = nullptr);
};

// ---- the reference's input objects of rtm_zero_op, without SEPlib ----

// Named parameters (Born/param_func.h): the operator reads bc_a (default 50),
// bc_b (0.0005), nbound (int(bc_a)) and rec_depth (0).  The reference's
// values come from the command line through SEPlib; here they are set in
// code.
class param_func {
 public:
  virtual ~param_func() {}
  virtual int get_int(const char *arg, int def) const;
  virtual float get_float(const char *arg, float def) const;
  param_func &set(const std::string &name, double value);
  std::map<std::string, double> vals;
};

// Velocity model on its grid (Born/vel_fd_3d.h), in host memory: every shot
// resamples it onto its padded grid with the random boundary.
class vel_fd_3d {
 public:
  vel_fd_3d(const std::vector<axis> &axes, const float *vel);
  axis get_axis(int iax) const { return axes[iax - 1]; }
  float max_vel() const;
  float min_vel() const;
  // the reference's rules, including dz returned when dy < dx
  // (Born/vel_fd_3d.h:11-26)
  float get_min_samp() const;
  float get_max_samp() const;
  std::vector<axis> axes;
  std::vector<float> vals;
};

// Source wavelet and shot positions (Born/source_func_3d.h).  The wavelet is
// given as recorded; its time derivative (Born/source_func_3d.cpp:4-20) is
// taken by the operator.
class source_func {
 public:
  source_func(axis at, const float *wavelet);
  // one shot per (sx, sy) node of the two axes at depth s_z, x fastest
  // (Born/source_func_3d.cpp:22-33)
  void set_sources_3d(float s_z, axis a_sx, axis a_sy);
  int get_points(bool) const { return 9; }
  float get_dt() const { return at.d; }
  axis get_axis(int) const { return at; }
  axis at;
  std::vector<float> wavelet, sx, sy, sz;
};

class data_rtm_3d;
class image_rtm_3d;

// The Born / RTM operator (Born/rtm_zero_op_3d.h).  Model: image on the model
// grid float[m3][m2][m1]; data: float[nshots][rny][rnx][data_nt].
class rtm_zero_op : public my_operator {
 public:
  explicit rtm_zero_op(const sepx_rtm_problem &p);
  // The reference's constructor (Born/rtm_zero_op_3d.cpp:8-36): the data
  // axes (t, receiver x, receiver y, shots ...) give the recording and the
  // receiver grid, the source the wavelet and the shot positions (one per
  // trace gather of `data`), the image the model grid (the operator's
  // domain is image->image, its range `data`).  do_src: propagate the
  // source wavefields now (else at the first adjoint); redo_src: propagate
  // them again at every adjoint.  aper, encode and rand_vec are accepted for
  // the signature: the reference's forward and adjoint do not use them.
  rtm_zero_op(param_func *par, vel_fd_3d *vel, source_func *source, data_rtm_3d *data,
              image_rtm_3d *image, float aper, bool verb, bool encode, int *rand_vec,
              bool do_src = true, bool redo_src = false);
  ~rtm_zero_op() override;
  bool forward(bool add, my_vector *model, my_vector *data, int iter = 1) override;
  bool adjoint(bool add, my_vector *model, my_vector *data, int iter = 1) override;
  void create_source_fields();   // mode 0: source_prop per shot, kept on the host
  hypercube_float *new_model() const;
  hypercube_float *new_data() const;
  struct shot_setup;
  struct impl;
  impl *d = nullptr;

 private:
  void init(const sepx_rtm_problem &p);
};

// Time mute (Born/tmute.h, Born/tmute.cpp:4-76): the samples of trace i2 from
// t_0 + x / vmute on (x = o2 + d2 i2, the axis-2 coordinate) pass, the earlier
// ones are removed.  Model and data: hypercube_float of the same shape, axes
// (t, x, ...).  forward of the reference moves its file cursor a whole cube per
// axis-3 index; here both directions apply the mask to every cube.
class tmute : public my_operator {
 public:
  tmute(float t, float v, my_vector *mod, my_vector *dat);
  bool forward(bool add, my_vector *model, my_vector *data, int iter = 1) override;
  bool adjoint(bool add, my_vector *model, my_vector *data, int iter = 1) override;
  float t_0, vmute;
};

// The image of a migration on its grid (Born/image_rtm_3d.h): sub-images
// (e.g. one shot's window) are added at the offset their origins give, and
// windows are read back through the mute.  mute == nullptr acts as 1.
class image_rtm_3d {
 public:
  explicit image_rtm_3d(const std::vector<axis> &axes);
  // the image on the velocity model's grid, zero (Born/image_rtm_3d.cpp:4-16)
  image_rtm_3d(const char *tag, const vel_fd_3d *vel);
  ~image_rtm_3d();
  void zero() { image->zero(); }
  void add(my_vector *v) { image->add(v); }
  image_rtm_3d(const image_rtm_3d &) = delete;
  void set_mute(const hypercube_float &m);          // copies m (same shape)
  void add_image(const hypercube_float *img);       // image_rtm_3d.cpp:24-49
  hypercube_float *extract_sub(axis a1, axis a2, axis a3) const;   // :52-90, caller owns it
  void write_volume();                              // image *= mute (:92-104)
  axis get_axis(int i) const { return image->get_axis(i); }
  hypercube_float *image = nullptr, *mute = nullptr;
};

// Multi-shot data (Born/data_rtm_3d.h): axes (t, x, y, shot); add_data
// accumulates one shot's traces (data_rtm_3d.cpp:37-51).
class data_rtm_3d : public hypercube_float {
 public:
  explicit data_rtm_3d(const std::vector<axis> &axes);
  // with the receiver depth parameter rec_depth (Born/data_rtm_3d.cpp:4-20)
  data_rtm_3d(const std::vector<axis> &axes, const param_func *par);
  void add_data(int ishot, const hypercube_float *dat);
  float sz = 0.f;   // receiver depth
  int nshots() const;   // product of the axes after the third
};

#endif /* __cplusplus */
#endif
