/*
 * sepx_oracle.h -- CPU restatement of SEP_Code's 3D acoustic Born/RTM path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity oracle for the CUDA
 * path in sep_code_gb300/ and the timed CPU baseline of bench.py.  Nothing in
 * the product links, imports or calls it.
 *
 * Every routine restates one piece of the reference (paths are relative to the
 * reference project root) with the reference's index ranges, step order and
 * quirks for the one-GPU case:
 *   Born/wave_fkernel.3d8o.cu   stencils, sponge, FD coefficients
 *   Born/gpu_funcs_3d.cu        inject / extract / imaging kernels, time loops
 *   Born/sinc_bob.cpp           8-tap least-squares sinc tables (Hale 1983)
 *   Born/vel_fd_3d.cpp          random-boundary velocity (glibc rand())
 *   Born/source_func_3d.cpp     padded domain, 9-point source stencil
 *   Born/data_rtm_3d.cpp        receiver geometry
 *   Born/map_data_3d.cpp, deriv_3d.cpp, laplac_3d.cpp   trace / image helpers
 *   Born/fd_prop_3d.cpp         stability dt
 *
 * Floating-point contract (shared with the CUDA kernels so that the two agree
 * bit for bit): every multiply-add that the reference writes as `a*b + c` is an
 * explicit fused multiply-add in a fixed order, everything else is an
 * individually rounded IEEE operation, denormals are kept.  The reference
 * builds with nvcc's default contraction and -ftz=true, whose exact rounding
 * pattern is compiler dependent; the differences are at the last-ulp level.
 *
 * Two precisions are exported: *_f32 (parity) and *_f64 (the precision oracle).
 */
#ifndef SEPX_ORACLE_H
#define SEPX_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* Padded propagation grid, axis 1 (x) fastest, axis 3 (z) slowest. */
typedef struct {
  int n1, n2, n3;
} orc_grid;

/* Everything the reference keeps in module globals / __constant__ symbols
 * (Born/gpu_finite_3d.h:31-86), passed explicitly. */
typedef struct {
  orc_grid g;
  float coeffs[13];          /* get_coeffs(d1,d2,d3) (wave_fkernel.3d8o.cu:26-27) */
  const float *damp_tab;     /* factor by sponge edge distance, 1.0 = no damping */
  int ntab;
  int ntrace;                /* ntrace_gpu: samples per trace (last transfer wins) */
  int nsinc;                 /* taps per sinc row (8) */
  const float *sinc_s;       /* source table  [ns][nsinc] */
  int ns;
  const float *sinc_d;       /* receiver table [nd][nsinc] */
  int nd;
  int nsrc;
  const int *src_loc;        /* linear cell index per source point */
  const float *src_vals;     /* [nsrc][ntrace] */
  int nrec_x, nrec_y;
  const int *rec_loc;        /* linear cell index per receiver */
} orc_ctx;

/* ---- set-up helpers (host math of the reference) ---- */
void orc_fd_coeffs(float d1, float d2, float d3, float out[13]);
/* table[e] = expf(-bc_b*(bc_a-e)) when < 1 else 1, e = 0..ntab-1 (f32 variant:
 * float argument, exponential rounded from double) */
void orc_damp_table_f32(float bc_a, float bc_b, int ntab, float *tab);
void orc_damp_table_f64(float bc_a, float bc_b, int ntab, double *tab);
void orc_sinc_table(int ntab, int nsinc, float *out /* [ntab][nsinc] */);
void orc_glibc_srand(unsigned int seed);
int orc_glibc_rand(void);
/* vel_fd_3d::rand_subspace.  model: (m1,m2,m3) with origins/spacings;
 * space: padded axes.  Writes (v+dev)^2*dt^2. */
void orc_rand_subspace(int irand, int nrand1, int nrand2, int nrand3, float dt,
                       const float *model, int m1, int m2, int m3,
                       float mo1, float mo2, float mo3, float md1, float md2, float md3,
                       int s1, int s2, int s3, float so1, float so2, float so3,
                       float sd1, float sd2, float sd3, float *out);
/* source_func::set_compute_size: padded sizes from model sizes */
void orc_compute_size(int m1, int m2, int m3, int nbt, int nb, int nby, int fat,
                      int *n1, int *n2, int *n3);
/* source_func::get_source_func: 9 source points, values [9][nts] */
void orc_source_func(const float *wavelet_deriv, int nwav, float sx, float sy, float sz,
                     int n1, int n2, float o1, float o2, float o3, float d1, float d2, float d3,
                     int nts, int *locs, float *vals);
/* wavelet time derivative done in source_func's constructor */
void orc_wavelet_deriv(const float *w, int n, float dt, float *out);
/* fd_prop::calc_stability: returns dt, writes nt */
float orc_calc_stability(float vmax, float dmin, float data_dt, int n_data, int *nt);
/* data_rtm_3d::get_source_func geometry + map_data ctor -> receiver cell indices */
void orc_receiver_map(int rnx, int rny, float ro2, float rd2, float ro3, float rd3, float rec_depth,
                      int n1, int n2, float o1, float o2, float o3, float d1, float d2, float d3,
                      int *locs);
/* deriv (time first difference of traces), laplac (z first difference), map_data */
void orc_deriv_forward(int add, int nt, int n2, int n3, float dt, const float *m, float *d);
void orc_deriv_adjoint(int add, int nt, int n2, int n3, float dt, float *m, const float *d);
void orc_laplac_forward(int add, int n1, int n2, int n3, const float *m, float *d);
void orc_laplac_adjoint(int add, int n1, int n2, int n3, float *m, const float *d);
void orc_map_data_forward(int add, int ntb, int nt, int n2, int n3, const float *m, float *d);
void orc_map_data_adjoint(int add, int ntb, int nt, int n2, int n3, float *m, const float *d);

/* ---- kernels (one call = one launch of the reference kernel) ---- */
void orc_wave_step_f32(const orc_ctx *c, int vel_inside, float *p0, const float *p1, const float *vel);
void orc_damp_f32(const orc_ctx *c, float *p0, float *p1);

/* ---- the three time loops of gpu_funcs_3d.cu (one GPU) ---- */
int orc_source_prop_f32(const orc_ctx *c, const float *vel, float *p0_out, float *p1_out,
                        int jt, int npts, int nt);
int orc_rtm_forward_f32(const orc_ctx *c, const float *vel, int jt, const float *img,
                        float *dat /* [nrec][ntrace] in/out */, int npts_src, int nt);
int orc_rtm_adjoint_f32(const orc_ctx *c, const float *vel, int jt, const float *p0_s,
                        const float *p1_s, float *img, const float *dat, int npts_src, int nt);

/* FP64 twins: every volume and trace in double, tables in double */
typedef struct {
  orc_ctx base;              /* geometry and trace sizes (its float coeffs are unused) */
  double d1, d2, d3;         /* grid spacings: coefficients are rebuilt in double */
  const double *damp_tab;
  const double *sinc_s, *sinc_d, *src_vals;
} orc_ctx64;
int orc_source_prop_f64(const orc_ctx64 *c, const double *vel, double *p0_out, double *p1_out,
                        int jt, int npts, int nt);
int orc_rtm_forward_f64(const orc_ctx64 *c, const double *vel, int jt, const double *img,
                        double *dat, int npts_src, int nt);
int orc_rtm_adjoint_f64(const orc_ctx64 *c, const double *vel, int jt, const double *p0_s,
                        const double *p1_s, double *img, const double *dat, int npts_src, int nt);

/* linearised Born pair with quantised source snapshots (prec 0 FP32, 1 BF16,
 * 2 FP16); snaps holds ceil(nt/js) full volumes */
int orc_lin_source_f32(const orc_ctx *c, const float *vel, int jt, int npts, int nt, int js,
                       int prec, float *snaps);
int orc_lin_forward_f32(const orc_ctx *c, const float *vel, int jt, int npts, int nt, int js,
                        int prec, const float *m, float *dat);
int orc_lin_adjoint_f32(const orc_ctx *c, const float *vel, int jt, int nt, int js,
                        const float *snaps, const float *dat, float *img);
int orc_lin_source_f64(const orc_ctx64 *c, const double *vel, int jt, int npts, int nt, int js,
                       double *snaps);
int orc_lin_forward_f64(const orc_ctx64 *c, const double *vel, int jt, int npts, int nt, int js,
                        const double *m, double *dat);
int orc_lin_adjoint_f64(const orc_ctx64 *c, const double *vel, int jt, int nt, int js,
                        const double *snaps, const double *dat, double *img);
/* source pass and adjoint in one call, the source wavefield recomputed from
 * checkpoints every seg steps instead of stored (same image as
 * orc_lin_source_* + orc_lin_adjoint_*; 2 ceil(nt/seg) + ceil(seg/js) + 7
 * volumes of memory) */
int orc_lin_adjoint_ckpt_f32(const orc_ctx *c, const float *vel, int jt, int npts, int nt, int js,
                             int prec, int seg, const float *dat, float *img);
int orc_lin_adjoint_ckpt_f64(const orc_ctx64 *c, const double *vel, int jt, int npts, int nt,
                             int js, int seg, const double *dat, double *img);

/* threads used by the OpenMP loops */
int orc_num_threads(void);
void orc_set_num_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
