/*
 * sepx.h -- C ABI of the GB300 (sm_103a) acoustic Born / RTM propagation path.
 *
 * Part 1 is a drop-in for the reference's GPU interface, Born/gpu_funcs_3d.h:4-27
 * of SEP_Code: the same eleven extern "C" functions with the same names,
 * argument order and meaning (host buffers in, host buffers out, one call runs
 * a whole time loop, module-global device state).  Like the reference they
 * return void; unlike the reference they never exit() the process: a failure
 * is recorded and can be read with sepx_last_error().
 *
 * Part 2 is the same interface with an int status (0 = success, negative =
 * error) under the sepx_ prefix, plus device-resident variants that keep the
 * image, traces and source wavefields in HBM between calls.
 *
 * Volumes are float[n3][n2][n1] (axis 1 fastest), traces float[nrec][ntrace],
 * exactly as the reference lays them out on the host.  One GPU (ngpus == 1);
 * the reference's multi-GPU z-slab split is not provided.
 */
#ifndef SEPX_H
#define SEPX_H
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- Part 1: reference-named C ABI ---------------- */

/* Born/gpu_funcs_3d.h:7 (gpu_funcs_3d.cu:10-45): select the device(s). */
void setup_cuda(int ngpus, int argc, char **argv);
/* Born/gpu_funcs_3d.h:9 (gpu_funcs_3d.cu:133-315): nt+1 steps of the source
 * wavefield with the random-boundary velocity; with get_last the last two
 * wavefields are returned in p0 (older) and p1 (newest).  `damp` is ignored,
 * as in the reference. */
void source_prop(int n1, int n2, int n3, bool damp, bool get_last, float *p0, float *p1, int jt,
                 int npts, int nt);
/* Born/gpu_funcs_3d.h:11 (gpu_funcs_3d.cu:509-712): receiver back-propagation,
 * source reconstruction from (p0_s_cpu, p1_s_cpu) and zero-lag image into img. */
void rtm_adjoint(int n1, int n2, int n3, int j, float *p0_s_cpu, float *p1_s_cpu, float *img,
                 int npts, int nt);
/* Born/gpu_funcs_3d.h:13 (gpu_funcs_3d.cu:317-505): Born modelling over img;
 * traces accumulate onto the receiver buffer given to transfer_receiver_func
 * and are returned in dat (nt_big samples per receiver). */
void rtm_forward(int n1, int n2, int n3, int jt, float *img, float *dat, int npts_src, int nt,
                 int nt_big, int nx, int ny);
/* Born/gpu_funcs_3d.h:15 (gpu_funcs_3d.cu:714-723): ns source sinc rows. */
void transfer_sinc_table_s(int nsinc, int ns, float **tables);
/* Born/gpu_funcs_3d.h:17 (gpu_funcs_3d.cu:725-733): ns receiver sinc rows. */
void transfer_sinc_table_d(int nsinc, int ns, float **tabled);
/* Born/gpu_funcs_3d.h:19 (gpu_funcs_3d.cu:735-745): source points (linear cell
 * index) and their traces float[npts][nt]. */
void transfer_source_func(int npts, int nt, int *locs, float *vals);
/* Born/gpu_funcs_3d.h:21 (gpu_funcs_3d.cu:747-758): receiver points and their
 * traces float[nx*ny][nt]. */
void transfer_receiver_func(int nx, int ny, int nt, int *locs, float *vals);
/* Born/gpu_funcs_3d.h:23 (gpu_funcs_3d.cu:761-767): v^2 dt^2 on the padded grid. */
void transfer_vel_func1(int nx, int ny, int nz, float *vel);
/* Born/gpu_funcs_3d.h:25 (gpu_funcs_3d.cu:769-775): second velocity; the
 * reference uploads it but no kernel reads it, so it is checked and dropped. */
void transfer_vel_func2(int nx, int ny, int nz, float *vel);
/* Born/gpu_funcs_3d.h:27 (gpu_funcs_3d.cu:777-803): grid spacing, sponge
 * (bc_a, bc_b) and padded grid; allocates the device volumes. */
void create_gpu_space(float d1, float d2, float d3, float bc_a, float bc_b, float bc_b_y, int nx,
                      int ny, int nz);

/* ---------------- Part 2: status-returning interface ---------------- */

int sepx_setup_cuda(int ngpus);
int sepx_create_gpu_space(float d1, float d2, float d3, float bc_a, float bc_b, float bc_b_y,
                          int nx, int ny, int nz);
int sepx_transfer_sinc_table_s(int nsinc, int ns, float **tables);
int sepx_transfer_sinc_table_d(int nsinc, int ns, float **tables);
int sepx_transfer_source_func(int npts, int nt, const int *locs, const float *vals);
int sepx_transfer_receiver_func(int nx, int ny, int nt, const int *locs, const float *vals);
int sepx_transfer_vel_func1(int nx, int ny, int nz, const float *vel);
/* receiver geometry with a zeroed device receiver buffer of nt samples */
int sepx_set_receivers(int nx, int ny, int nt, const int *locs);
int sepx_transfer_vel_func2(int nx, int ny, int nz, const float *vel);
int sepx_source_prop(int n1, int n2, int n3, bool damp, bool get_last, float *p0, float *p1,
                     int jt, int npts, int nt);
int sepx_rtm_forward(int n1, int n2, int n3, int jt, const float *img, float *dat, int npts_src,
                     int nt, int nt_big, int nx, int ny);
int sepx_rtm_adjoint(int n1, int n2, int n3, int jt, const float *p0_s, const float *p1_s,
                     float *img, int npts, int nt);

/* Device-resident variants: enqueue the time loop on the context stream and
 * return without synchronising.  source_prop keeps its last two wavefields in
 * HBM; rtm_forward reads the image set by sepx_set_image and accumulates into
 * the receiver buffer; rtm_adjoint images into the image buffer, starting
 * from the last source_prop wavefields read back swapped as rtm_zero_op does
 * (use_source_last != 0) or from the ones set with sepx_set_source_fields. */
int sepx_source_prop_resident(int jt, int npts, int nt);
int sepx_rtm_forward_resident(int jt, int npts_src, int nt);
int sepx_rtm_adjoint_resident(int jt, int npts, int nt, int use_source_last);
/* Linearised Born pair (the operator of least-squares RTM, rtm_zero_op's
 * forward/adjoint): the source pass stores the source wavefield every js steps
 * (prec 0 = FP32, 1 = BF16, 2 = FP16 with a power-of-two max-abs scale per
 * 32x16 block of each plane); the forward scatters from the image buffer
 * into the receiver buffer with the same stored values, recomputing the
 * source field; the adjoint images the receiver buffer into the image buffer.
 * Forward and adjoint are exact transposes of each other (up to FP32
 * rounding), unlike the reference's rtm_forward / rtm_adjoint pair. */
int sepx_lin_source_pass(int jt, int npts, int nt, int js, int prec);
int sepx_lin_forward_resident(int jt, int npts, int nt, int js, int prec);
int sepx_lin_adjoint_resident(int jt, int nt, int js, int prec);
long long sepx_snapshot_bytes(int nt, int js, int prec);
int sepx_set_image(const float *img);                 /* host, dense */
int sepx_get_image(float *img);                       /* host, dense */
int sepx_set_source_fields(const float *p0, const float *p1);
int sepx_get_source_fields(float *p0, float *p1);
int sepx_set_traces(const float *vals);               /* [nrec][ntrace] */
int sepx_get_traces(float *vals);
int sepx_zero_traces(void);                          /* receiver buffer := 0 on the device */
int sepx_synchronize(void);
void *sepx_get_stream(void);          /* the cudaStream_t every call enqueues on */

/* FP64-accumulated dot product of two device float vectors (b == NULL: the
 * sum of a), as my_vector::dot (Born/hypercube_float.cpp:123-133); the result
 * is written to host memory; synchronous. */
int sepx_dot_f32(const float *a, const float *b, long long n, double *result);

/* No counterpart in the reference.  The same FP64 dot product with no device
 * allocation by the library, for callers that cannot let a library allocate
 * device memory (services that reserve their whole device-memory budget at
 * start-up, hosts whose own pool owns every allocation).  a, b (b == NULL: the
 * sum of a) and d_result are device pointers owned by the caller; the work is
 * enqueued on `stream` (a cudaStream_t; NULL = the default stream) and
 * d_result is valid once the stream reaches it.  Scratch is a fixed 256 KB
 * file-scope device array held by every GPU that loads the library: n may be
 * at most sepx_dot_f32_noalloc_max_elems() (268,435,456) elements, larger
 * calls are rejected.  All calls share that array; calls that overlap on the
 * GPU race on it.  The first call on a device looks up the array's address
 * with that device current and should come before any stream capture; the
 * address is kept for the device's primary context, so the function assumes
 * that context (no cudaDeviceReset after the first call, no other context on
 * the same device).  NULL b sums a; n = 0 writes 0 to d_result. */
int sepx_dot_f32_noalloc(const float *a, const float *b, long long n, double *d_result,
                         void *stream);
long long sepx_dot_f32_noalloc_max_elems(void);

/* Per-shot glue of the operator layer, on the context's buffers:
 * image_to_padded: image buffer := laplac(extract_sub(model)) (model is a
 *   device float[m3][m2][m1]; model cell = padded cell + (f1,f2,f3));
 * padded_to_image: model += add_image(laplac'(image buffer));
 * traces_to_data:  data += deriv(map_data(receiver buffer)) (device
 *   float[nrec][nt], nt data samples of spacing dt);
 * data_to_traces:  receiver buffer := map_data'(deriv'(data)).
 * (Born/rtm_zero_op_3d.cpp:139-166, :248-274 and the helpers they call.) */
int sepx_op_image_to_padded(const float *model, int m1, int m2, int m3, int f1, int f2, int f3);
int sepx_op_padded_to_image(float *model, int m1, int m2, int m3, int f1, int f2, int f3);
int sepx_op_traces_to_data(float *data, int nt, float dt);
int sepx_op_data_to_traces(const float *data, int nt, float dt);

/* Image and data vectors kept in HBM, on the context stream (the reference
 * keeps them in out-of-core SEP files and loops over them on the host):
 * image_add_window:     image_rtm_3d::add_image (Born/image_rtm_3d.cpp:24-49):
 *   img[n3][n2][n1] cell j + f += sub[s3][s2][s1] cell j, where inside img;
 * image_extract_window: image_rtm_3d::extract_sub (:52-90): sub cell j =
 *   img * mute at j + f (mute NULL: 1), 0 outside img;
 * tmute:                tmute::forward / adjoint (Born/tmute.cpp:4-76) on
 *   [nrep][n2][n1] traces: data (+)= model (adj: model (+)= data) from sample
 *   (int)((t0 + (o2 + d2 i2) / vmute - o1) / d1) of trace i2 on (a start
 *   before the first sample is taken as 0); add = 0 zeroes the output first.
 * All buffers are device pointers. */
int sepx_image_add_window(float *img, int n1, int n2, int n3, int f1, int f2, int f3,
                          const float *sub, int s1, int s2, int s3);
int sepx_image_extract_window(const float *img, const float *mute, int n1, int n2, int n3, int f1,
                              int f2, int f3, float *sub, int s1, int s2, int s3);
int sepx_tmute(int adj, int add, float t0, float vmute, int n1, float o1, float d1, int n2, float o2,
               float d2, long long nrep, float *model, float *data);

/* Device float vectors and BLAS-1 on the context stream (hypercube_float,
 * Born/hypercube_float.cpp:123-223; scale factors applied in double). */
int sepx_vec_alloc(float **p, long long n);
int sepx_vec_free(float *p);
int sepx_vec_upload(float *d, const float *h, long long n);
int sepx_vec_download(float *h, const float *d, long long n);
int sepx_vec_copy(float *dst, const float *src, long long n);
int sepx_vec_fill(float *x, long long n, float v);
int sepx_vec_scale(float *y, long long n, double a);
int sepx_vec_scale_add(float *y, const float *x, long long n, double a, double b); /* y = a y + b x */
int sepx_vec_scale_add2(float *y, const float *x1, const float *x2, long long n, double a,
                        double b);                                                /* y = a x1 + b x2 */
int sepx_vec_add(float *y, const float *x, long long n);
int sepx_vec_mult(float *y, const float *x, long long n);
int sepx_vec_random(float *y, long long n, unsigned long long seed);   /* uniform(-0.5, 0.5) */

/* Diagnostics and tuning. */
const char *sepx_last_error(void);
int sepx_device_error(void);          /* device error word (bounded waits), then cleared */
long long sepx_kernel_launches(void); /* kernels launched by this library so far */
int sepx_set_zchunk(int planes);      /* z planes per CTA; 0 = automatic */
/* Rows per consumer thread of a step kernel (tuning knob): mode 0 =
   source_prop, 1 = Born forward, 2 = RTM adjoint steps; rows 1 (tile 32 x 16,
   the default) or 2 (tile 32 x 32).  Both give identical results. */
int sepx_set_tile_rows(int mode, int rows);
int sepx_reset(void);                 /* free every device buffer */

#ifdef __cplusplus
}
#endif
#endif
