/*
 * sepx_unet.h -- kernels of the learned preconditioner for least-squares RTM:
 * a 3-D U-Net whose convolutions run as BF16 implicit GEMMs on the tcgen05
 * tensor cores with FP32 accumulation in tensor memory.
 *
 * No counterpart in the reference: these are the building blocks of the
 * direction preconditioner applied where the reference's solver forms the
 * search direction (Born/lin_solver.cpp:127-128) and where its vectors
 * offer an inverse-Hessian hook (Born/my_vector.h:41).
 *
 * Conventions: device pointers; activations are channel-last BF16 volumes
 * [nb][D][H][W][cstride] read or written at channel offset coff (channel
 * counts, strides and offsets multiples of 8); `stream` is a cudaStream_t
 * (NULL = the legacy stream).  Every call returns 0 or -1 with the reason in
 * sepx_last_error().
 */
#ifndef SEPX_UNET_H
#define SEPX_UNET_H

#ifdef __cplusplus
extern "C" {
#endif

/* Master weights are FP32 [ntap][cin_p][cout] (cin_p = input channels
 * rounded up to 8; row t*cin_p + c), the layout the weight gradient has.
 * BF16 elements of the packed operand (transpose 0: forward, cout outputs;
 * 1: data gradient, cin_p outputs, taps flipped) */
int sepx_unet_packed_elems(int cout, int cin_p, int ntap, int transpose);
int sepx_unet_pack_weights(const float *w, int cout, int cin_p, int ntap, int transpose, void *out,
                           void *stream);
/* njobs (<= 64) packings in one launch; the arrays are host arrays of
 * length njobs, job i as sepx_unet_pack_weights(w[i], cout[i], cin_p[i],
 * ntap[i], transpose[i], out[i]) */
int sepx_unet_pack_weights_many(int njobs, const float *const *w, void *const *out, const int *cout,
                                const int *cin_p, const int *ntap, const int *transpose, void *stream);
/* y = act(conv(x, w) + bias), ntap 27 (3x3x3, zero padding 1) or 1 (1x1x1),
 * cin = channels read from x (a multiple of 8); y (BF16 view) and/or yf
 * (FP32 [voxels][cout], plus resid[voxels][cout] when resid is not NULL) */
int sepx_unet_conv_fwd(const void *x, int x_cstride, int x_coff, int nb, int D, int H, int W, int cin,
                       int ntap, const void *wpacked, const float *bias, int cout, int relu, void *y,
                       int y_cstride, int y_coff, float *yf, const float *resid, void *stream);
/* The same with the ReLU backward fused into the epilogue (for the data
 * gradient): outputs become 0 where the BF16 view mask (cout channels at
 * mask_coff) is not > 0 -- bit-identical to sepx_unet_relu_mask afterwards.
 * mask NULL: no mask.  cout must be a multiple of 8 when mask is given. */
int sepx_unet_conv_fwd_masked(const void *x, int x_cstride, int x_coff, int nb, int D, int H, int W,
                              int cin, int ntap, const void *wpacked, const float *bias, int cout, int relu,
                              void *y, int y_cstride, int y_coff, float *yf, const float *resid,
                              const void *mask, int mask_cstride, int mask_coff, void *stream);
/* 3x3x3 layers whose planes are at least 16 x 8 voxels and whose packed
 * weights and input halo fit in 227 KB of shared memory run on the
 * halo-staged kernel, and the weight gradients of 3x3x3 layers with at most
 * 40 output and 80 input channels on the TMA-staged tap-stacked kernel;
 * enable = 0 sends every layer to the per-tap gather kernels.  Returns the
 * previous setting. */
int sepx_unet_set_halo(int enable);
/* Weight-gradient kernel choice (with the halo-staged kernels enabled):
 * 2 (default) the z-walk tap-stacked kernel (cin <= 48, cout <= 40), else
 * the per-tile tap-stacked kernel (cin <= 80, cout <= 40), else the gather
 * kernel; 1 the per-tile kernel, else gather; 0 gather.  Returns the
 * previous choice, or -1 for another value. */
int sepx_unet_set_wgrad_form(int form);
/* dw[t*cin + c][cout] += sum_v x[v + off(t)][c] dy[v][cout]  (FP32
 * accumulation); dy holds cout rounded up to 8 channels at dy_coff */
int sepx_unet_conv_wgrad(const void *x, int x_cstride, int x_coff, int nb, int D, int H, int W,
                         int cin, int ntap, const void *dy, int dy_cstride, int dy_coff, int cout,
                         float *dw, void *stream);
/* The same, plus db[cout] += sum_v dy[v][cout] when db is not NULL (taken
 * from the same tiles on the tap-stacked kernel).  The tap-stacked kernel
 * sums per-CTA partials in a fixed order (repeatable results); it keeps them
 * in a library scratch buffer per stream (up to 16 streams), grown on demand:
 * the first call of a shape on a stream must not be inside a graph capture. */
int sepx_unet_conv_wgrad_bias(const void *x, int x_cstride, int x_coff, int nb, int D, int H, int W,
                              int cin, int ntap, const void *dy, int dy_cstride, int dy_coff, int cout,
                              float *dw, float *db, void *stream);
/* 2x2x2 average pooling and its gradient (accumulate 1: dx += ...) */
int sepx_unet_avgpool(const void *x, int x_cstride, int x_coff, int nb, int D, int H, int W, int c,
                      void *y, int y_cstride, int y_coff, void *stream);
int sepx_unet_avgpool_bwd(const void *dy, int dy_cstride, int dy_coff, int nb, int D, int H, int W,
                          int c, void *dx, int dx_cstride, int dx_coff, int accumulate, void *stream);
/* ... then dx = 0 where the BF16 view mask is not > 0 (the ReLU backward of
 * the layer that produced dx's activation, applied after the sum) */
int sepx_unet_avgpool_bwd_masked(const void *dy, int dy_cstride, int dy_coff, int nb, int D, int H, int W,
                                 int c, void *dx, int dx_cstride, int dx_coff, int accumulate,
                                 const void *mask, int mask_cstride, int mask_coff, void *stream);
/* nearest x2 upsampling of a (D, H, W) volume and its gradient */
int sepx_unet_upsample(const void *x, int x_cstride, int x_coff, int nb, int D, int H, int W, int c,
                       void *y, int y_cstride, int y_coff, void *stream);
int sepx_unet_upsample_bwd(const void *dy, int dy_cstride, int dy_coff, int nb, int D, int H, int W,
                           int c, void *dx, int dx_cstride, int dx_coff, void *stream);
int sepx_unet_upsample_bwd_masked(const void *dy, int dy_cstride, int dy_coff, int nb, int D, int H, int W,
                                  int c, void *dx, int dx_cstride, int dx_coff, const void *mask,
                                  int mask_cstride, int mask_coff, void *stream);
/* dy = 0 where y <= 0 (ReLU backward, in place) */
int sepx_unet_relu_mask(const void *y, int y_cstride, int y_coff, void *dy, int dy_cstride,
                        int dy_coff, long long V, int c, void *stream);
/* db[c] += sum over voxels of dy[v][c] */
int sepx_unet_bias_grad(const void *dy, int dy_cstride, int dy_coff, long long V, int c, float *db,
                        void *stream);
/* FP32 single-channel volume * scale -> channel coff of a BF16 view (8-channel group, rest 0) */
int sepx_unet_to_bf16(const float *in, long long V, float scale, void *y, int y_cstride, int y_coff,
                      void *stream);
/* *loss += mean (out - target)^2 (FP64); g (BF16, channel 0 of 8) = d loss / d out */
int sepx_unet_mse(const float *out, const float *target, long long V, void *g, int g_cstride,
                  double *loss, void *stream);
/* Adam step on FP32 parameters (step counts from 1) */
int sepx_unet_adam(float *p, const float *g, float *m, float *v, long long n, float lr, float b1,
                   float b2, float eps, int step, void *stream);
/* The same step with its hyper-parameters read from device memory when the
 * kernel runs: hp = {lr, b1, b2, eps, step} (FP32; step counts from 1, exact
 * below 2^24), so that a captured training step replays with the current
 * learning rate and step count.  A step below 1 makes no update and sets the
 * status word (sepx_unet_status() == 5). */
int sepx_unet_adam_dev(float *p, const float *g, float *m, float *v, long long n, const float *hp,
                       void *stream);
/* CUDA-graph capture of the calls this thread enqueues on `stream` (not the
 * legacy stream) between begin and end; end instantiates the graph and
 * returns its handle, launch replays it on a stream, free releases it.
 * Nothing may synchronise or allocate between begin and end: run the
 * captured sequence once without capture first. */
int sepx_unet_capture_begin(void *stream);
int sepx_unet_capture_end(void *stream, void **graph);
int sepx_unet_graph_launch(void *graph, void *stream);
int sepx_unet_graph_free(void *graph);
/* device status word of the convolution kernels (0 = no bounded wait gave up) */
int sepx_unet_status(void);

#ifdef __cplusplus
}
#endif
#endif
