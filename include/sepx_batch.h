/*
 * sepx_batch.h -- many shots per time step.
 *
 * The reference models its shots one after another: rtm_zero_op's shot loop
 * (Born/rtm_zero_op_3d.cpp:123) sets up each shot through the C ABI of
 * Born/gpu_funcs_3d.h and runs rtm_forward.  A batch keeps one device context
 * per shot: after sepx_batch_select(i) the ordinary calls of include/sepx.h
 * (create_gpu_space, transfer_*, sepx_set_image, ...) set up or read shot i.
 * sepx_batch_rtm_forward then advances the Born forward of every shot at
 * once.  No counterpart in the reference beyond that shot loop.
 */
#ifndef SEPX_BATCH_H
#define SEPX_BATCH_H

#ifdef __cplusplus
extern "C" {
#endif

/* nshots empty contexts (setup_cuda first); ends any previous batch */
int sepx_batch_begin(int nshots);
/* make shot i the target of the C ABI; -1 returns to the single context */
int sepx_batch_select(int ishot);
int sepx_batch_size(void);
int sepx_batch_end(void);
/* Born forward (rtm_forward semantics: image set with sepx_set_image,
 * traces accumulated into each shot's receiver buffer) of every shot, nt
 * steps.  how 0: shot after shot, one launch per step and shot; 1: one launch
 * per step for all shots, in the tuned style (0: a grid of every shot's
 * tiles, parameter sets in parameter space; 1: a persistent grid walking a
 * list of (shot, tile, z-chunk) items); 2: those launches captured into a
 * CUDA graph once and replayed (re-captured when nt, jt or the tuning
 * change).  Every shot must use the same jt and nt. */
int sepx_batch_rtm_forward(int jt, int npts_src, int nt, int how);
/* the same for source_prop (nt + 1 steps; the two last fields kept per shot)
 * and for rtm_adjoint on those fields (sepx_rtm_adjoint_resident semantics
 * with use_source_last = 1: image per shot via sepx_get_image) */
int sepx_batch_source_prop(int jt, int npts, int nt, int how);
int sepx_batch_rtm_adjoint(int jt, int npts, int nt, int how);
/* time nsteps batched steps for every style x z-chunk x ring-depth candidate,
 * keep the fastest (clears every shot's receiver traces) */
int sepx_batch_autotune(int jt, int npts_src, int nsteps, int *zchunk, int *stages, int *style,
                        float *best_ms);
/* zchunk 0: the single-shot default; stages 2, 3 or 4; style 0 or 1 */
int sepx_batch_set_tuning(int zchunk, int stages, int style);
int sepx_batch_get_tuning(int *zchunk, int *stages, int *style);

#ifdef __cplusplus
}
#endif
#endif
