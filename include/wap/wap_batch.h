/* wap_batch.h -- the batched form: several independent scans of uneven sizes
 * (each a wap_ctx with its time level set up and its projections loaded)
 * reconstructed together on one GPU.
 *
 * One outer iteration of the batch is, for every scan, exactly
 * wap_outer_iteration on its context (same kernels, same bits), arranged so
 * that the GPU is filled by all scans at once: in each Chambolle-Pock
 * iteration the SART steps of every frame of every scan run as one persistent
 * work-queue launch per step for the forward projections and one for the
 * backprojections (blocks take (scan, tile) items from a counter), the whole
 * CP iteration is captured once as a CUDA graph and replayed; the flows and
 * the warp-and-project pass of the scans run concurrently on the scans' own
 * streams.  The work-queue kernels' tile shapes (pixels per projector block,
 * voxels per backprojector block) are picked by timing them on the batch's
 * largest step, unless set.  Observers (wap_set_observer) are not called for
 * the batch's CP iterations.  The reference reconstructs one scan per
 * process; this layer has no counterpart there.
 */
#ifndef WAP_WAP_BATCH_H
#define WAP_WAP_BATCH_H

#include "wap/wap.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct wap_batch wap_batch;

/* ctxs: n contexts on one device, each with a level set up
 * (wap_level_setup) and projections uploaded; the batch borrows them (they
 * must outlive it and not be used by other threads while it runs). */
WAP_API int wap_batch_create(wap_batch **out, wap_ctx *const *ctxs, int n);
WAP_API void wap_batch_destroy(wap_batch *b);
WAP_API const char *wap_batch_last_error(const wap_batch *b);
/* One outer iteration of every scan: scheds[i] is scan i's schedule; all
 * share n_cp, nb_sart and bp_exact (the merged CP iterations need them
 * equal).  stats (may be NULL) receives the sums over the scans, with ms_cp
 * the whole batch's device time. */
WAP_API int wap_batch_outer_iteration(wap_batch *b, const wap_schedule *scheds, wap_stats *stats);
/* Tile shapes of the work-queue kernels: fp 0 = 16x8 pixels per block,
 * 1 = 8x8, 2 = 32x8; bp 0 = 32x4x2 voxels, 1 = 32x8x1, 2 = 32x2x4; -1 =
 * autotuned (the default).  Every shape gives the same results. */
WAP_API int wap_batch_set_tuning(wap_batch *b, int fp_shape, int bp_shape);
WAP_API int wap_batch_get_tuning(const wap_batch *b, int *h_fp_shape, int *h_bp_shape);

#ifdef __cplusplus
}
#endif
#endif /* WAP_WAP_BATCH_H */
