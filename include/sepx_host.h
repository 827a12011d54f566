/*
 * sepx_host.h -- host set-up math of the Born/RTM operator (sep_code_gb300).
 * Each function restates the reference's host code that prepares the inputs
 * of the GPU C ABI (include/sepx.h) for one shot; values are identical to the
 * reference's bit for bit.
 */
#ifndef SEPX_HOST_H
#define SEPX_HOST_H
#ifdef __cplusplus
extern "C" {
#endif

/* sinc_bob(ntab, nsinc) tables, Born/sinc_bob.cpp:4-40: out[ntab][nsinc] */
void sepx_host_sinc_table(int ntab, int nsinc, float *out);
/* the first n values of srand(seed); rand() (glibc's additive generator) */
int sepx_host_glibc_rand_sequence(unsigned int seed, int n, int *out);
/* vel_fd_3d::rand_subspace, Born/vel_fd_3d.cpp:26-88: v^2 dt^2 on the padded
 * grid (s1,s2,s3) from the model (m1,m2,m3) with a random boundary */
void sepx_host_rand_subspace(int irand, int nrand1, int nrand2, int nrand3, float dt,
                             const float *model, int m1, int m2, int m3, float mo1, float mo2,
                             float mo3, float md1, float md2, float md3, int s1, int s2, int s3,
                             float so1, float so2, float so3, float sd1, float sd2, float sd3,
                             float *out);
/* source_func::set_compute_size, Born/source_func_3d.cpp:37-64 */
void sepx_host_compute_size(int m1, int m2, int m3, int nbt, int nb, int nby, int fat, int *n1,
                            int *n2, int *n3);
/* wavelet time derivative, Born/source_func_3d.cpp:4-19 */
void sepx_host_wavelet_deriv(const float *w, int n, float dt, float *out);
/* source_func::get_source_func, Born/source_func_3d.cpp:100-133 */
void sepx_host_source_func(const float *wav, int nwav, float sx, float sy, float sz, int n1, int n2,
                           float o1, float o2, float o3, float d1, float d2, float d3, int nts,
                           int *locs, float *vals);
/* fd_prop::calc_stability, Born/fd_prop_3d.cpp:7-26: returns dt, writes nt */
float sepx_host_calc_stability(float vmax, float dmin, float data_dt, int n_data, int *nt);
/* receiver cells, Born/data_rtm_3d.cpp:115-140 + Born/map_data_3d.cpp:4-35 */
void sepx_host_receiver_map(int rnx, int rny, float ro2, float rd2, float ro3, float rd3,
                            float rec_depth, int n1, int n2, float o1, float o2, float o3, float d1,
                            float d2, float d3, int *locs);

#ifdef __cplusplus
}
#endif
#endif
