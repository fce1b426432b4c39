/* wap.h -- C ABI of the GB300-native warp-and-project (WaP) reconstruction
 * hot path.
 *
 * The reference (WaP19) exposes its hot path as C++ entry points, not as an
 * FFI; each function below replaces one of them, named in its comment with
 * the reference file:line it stands in for.  Arguments are plain pointers and
 * sizes.  Array layouts follow the reference's CImg images: idx = x + W*(y +
 * H*z), channels planar (a 3-component flow is three consecutive volumes).
 *
 * Pointer kinds: arguments named h_* are host memory, d_* are device memory
 * on the context's device.  Every call returns WAP_OK or a WAP_E* status and
 * never throws; wap_last_error() gives the message of the last failure on that
 * context.  A context is used by one host thread at a time; work is ordered on
 * the context's stream (wap_set_stream), and calls that return host data
 * synchronise that stream.
 */
#ifndef WAP_WAP_H
#define WAP_WAP_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WAP_API __attribute__((visibility("default")))

enum {
  WAP_OK = 0,
  WAP_EINVAL = 1,   /* bad argument or size */
  WAP_ENOMEM = 2,   /* device or host allocation failed */
  WAP_ECUDA = 3,    /* CUDA runtime error */
  WAP_ESTATE = 4,   /* call out of order (e.g. no level set up) */
  WAP_ENODEV = 5,   /* no usable GPU */
  WAP_ETOOBIG = 6,  /* problem larger than a fixed-capacity entry point allows */
  WAP_EHOST = 8     /* other host-side failure (e.g. a worker thread could not start); 7 is WAP_EIO */
};

typedef struct wap_ctx wap_ctx;

/* Scan geometry and solver weights: the reference's command-line options
 * (main.cpp:15-138) plus the projection count it hard-codes (main.cpp:198). */
typedef struct {
  int vol[3];       /* -f  volume dims */
  int det[2];       /* -u  detector W, H */
  int nproj;        /* projections in the stack (main.cpp:198) */
  int nframes_cli;  /* -v  frames at time level 0 */
  double vs;        /* -c  voxel spacing */
  double ds;        /* -d  detector spacing */
  double sid;       /* -g  source to iso-centre distance */
  double sdd;       /* -j  source to detector distance */
  double oxyz[3];   /* --oxyz  volume centre offset */
  double alpha;     /* -a  SART relaxation */
  double tv_w;      /* -s  spatial TV weight */
  double tp_w;      /* -t  temporal weight */
} wap_scan_desc;

/* One outer iteration's schedule (WaP_Tomo.cpp:478-492, 711-727). */
typedef struct {
  int n_cp;          /* Chambolle-Pock iterations (nb_volOpt[level]) */
  int nb_sart;       /* SART sweeps per proximal call (nb_proxiSART) */
  int nb_projwarp;   /* warp-and-project passes (nb_projwarp) */
  int wp_frames;     /* frames the WaP pass visits (WaP_Tomo.cpp:801) */
  float flow_tol;    /* 0.008 */
  float flow_lambda; /* 0.05 */
  int flow_iters;    /* 3000 */
  int flow_warps;    /* 3 */
  float flow_eta;    /* 0.5 */
  float flow_sigma;  /* 0.8 */
  int flow_scales;   /* 5 */
  int cut;           /* ROI margin, 8 */
  int bp_exact;      /* 1: bicubic BP in the reference's double arithmetic; 0: FP32 FMA */
} wap_schedule;

/* Counters of the last outer iteration (reset by each wap_outer_iteration*). */
typedef struct {
  long long flow_pd_iterations;  /* primal-dual iterations over all pairs, levels, warps */
  long long fp_launches;
  long long kernel_launches;     /* every kernel this library launched */
  double ms_cp, ms_flow, ms_wap; /* device time per phase (CUDA events) */
  double pd_voxel_iters;         /* sum over PD iterations of the level's voxel count */
  double advect_voxels;          /* voxels warped (all advect calls) */
  long long projections;         /* forward projections (one per frame job) */
  long long backprojections;     /* voxel-driven backprojections */
  long long cp_frame_passes;     /* CP dual + primal + over-relaxation, per frame */
  double ms_pd;                  /* profiled: device time of the PD iterations at the largest grid */
  long long pd_timed;            /* profiled: PD iterations in ms_pd */
  long long pd_timed_voxels;     /* profiled: voxels of that grid */
  /* per flow pyramid level, index 0 = finest: device time of the level's
   * solve (warps, linearisations, primal-dual iterations) and its
   * primal-dual iterations, summed over the pairs */
  double ms_flow_level[8];
  long long pd_iters_level[8];
} wap_stats;

/* ---- context ---------------------------------------------------------- */

/* Builds VolumeData + PSART state for a scan (main.cpp:195-219,
 * WaP_Tomo.cpp:228-434): per-projection geometry (PSART::RotateVolume +
 * Scene/_calculateMatrix, WaP_Tomo.cpp:1764-1797) is computed once here.
 * h_angles_deg: nproj angles in degrees (WaP_Tomo.cpp:324-331). */
WAP_API int wap_create(wap_ctx **out, const wap_scan_desc *scan, const double *h_angles_deg, int device);
WAP_API void wap_destroy(wap_ctx *ctx);
WAP_API const char *wap_last_error(const wap_ctx *ctx);
WAP_API int wap_set_stream(wap_ctx *ctx, void *cuda_stream);
WAP_API int wap_synchronize(wap_ctx *ctx);
WAP_API int wap_get_stats(wap_ctx *ctx, wap_stats *out);
/* 1: time primal-dual iterations of the flow solver at the largest grid with
 * CUDA events on the context's stream (every tenth launch, so the others
 * keep their programmatic overlap; wap_stats.ms_pd / pd_timed is the mean
 * launch time); 0 (default): no per-launch events. */
WAP_API int wap_set_profiling(wap_ctx *ctx, int on);

/* A context without a scan, for the calls that take their grid as arguments
 * (wap_advect, wap_blur, wap_resize, wap_flow_level, wap_flow_multiscale,
 * wap_cg_screened_laplacian and the memory helpers below);
 * the scan-dependent calls return WAP_ESTATE on it. */
WAP_API int wap_create_compute(wap_ctx **out, int device);

/* Device memory of destroyed contexts is kept in a process-wide cache and
 * reused by later contexts (cudaFree would synchronise the whole device).
 * wap_cached_bytes: bytes held there; wap_trim_cache(device): frees them
 * (device < 0: all devices) and returns the bytes freed.  A failed
 * allocation empties the cache of its device and retries by itself. */
WAP_API size_t wap_cached_bytes(void);
WAP_API size_t wap_trim_cache(int device);

/* Device memory helpers, so that callers need no CUDA headers: allocation on
 * the context's device, and copies ordered on the context's stream that
 * return when the copy is complete. */
WAP_API int wap_alloc(wap_ctx *ctx, size_t bytes, void **d_out);
WAP_API int wap_free(wap_ctx *ctx, void *d_ptr);
WAP_API int wap_copy_to_device(wap_ctx *ctx, void *d_dst, const void *h_src, size_t bytes);
WAP_API int wap_copy_to_host(wap_ctx *ctx, void *h_dst, const void *d_src, size_t bytes);
WAP_API int wap_fill_zero(wap_ctx *ctx, void *d_ptr, size_t bytes);

/* Observer of the solver's intermediate states, the points at which the
 * reference writes its Analyze dumps:
 *   WAP_EV_SART  after the SART proximal operator of frame a in CP iteration b
 *                (b = 1..n_cp), d_data = the frame's volume
 *                (WaP_Tomo.cpp:1669);
 *   WAP_EV_FLOW  after the flow of the pair (a, a+1), d_data = frame a's
 *                3-channel flow (WaP_Tomo.cpp:764-771);
 *   WAP_EV_WARP  after the warp-and-project step of frame a at projection b,
 *                d_data = the frame's volume (WaP_Tomo.cpp:1417-1418).
 * The call comes from the thread running the outer iteration, after the
 * context's stream has finished the step; d_data is valid only during the
 * call.  The observer may use the device-pointer calls and the memory helpers
 * on the same context (e.g. wap_advect, wap_copy_to_host) but not the solver
 * calls (wap_sart_prox, wap_warp_and_project, wap_outer_iteration*).  Frames
 * that the library batches into one launch report one event each, in frame
 * order, after that launch; each event's data is the state the reference
 * dumps at that point.  Results are identical with or without an observer.
 * fn = NULL removes it. */
enum { WAP_EV_SART = 1, WAP_EV_FLOW = 2, WAP_EV_WARP = 3 };
typedef void (*wap_observer_fn)(void *user, int event, int level, int a, int b, const float *d_data);
WAP_API int wap_set_observer(wap_ctx *ctx, wap_observer_fn fn, void *user);

/* Kernel-shape choices (results are identical for every choice; only speed
 * changes).  key "pd_form": 0 = autotuned per grid size (default), 1 = the
 * fused primal-dual kernel, 2 = the primal + dual kernel pair, 3 = the
 * TMA-fed fused kernel (grids with nx % 4 == 0, else 2); "pd_zchunk": z
 * planes per block, 0 = autotuned / default; "fp_bricks": 1 (default) = the
 * forward projector reads a 4x4x4 brick-layout copy of each volume, 0 = the
 * linear volume.  "flow_lanes": an outer iteration's flow pairs run
 * concurrently on this many lanes (helper contexts with their own streams
 * and workspaces; each pair's flow is the one it gets alone), 1 = one pair
 * after another, up to 8; 0 (default) = automatic: 4 lanes for volumes of at
 * most 128^3 voxels, whose flow levels are latency-bound, 2 above.  "bp_ray": 0 (default) = SART backprojects voxel-driven
 * with the reference's bicubic weights; 1 = SART backprojects with the
 * matched ray-driven splat (the ray caster's back-projection mode,
 * SingleScalarVolume.core.h:85-96,149-199, which the reference's
 * --bp Raybased allocates sums for, TypicalRayProducer.cpp:42-45,100-104)
 * and updates vol += alpha * contribution / weight where weight > 0, then
 * clamps to [0, G_Max] (column-sum normalisation); warp-and-project keeps
 * the voxel-driven backprojection.  "splat_form": 0 (default) = the
 * ray-driven splat accumulates each slab of a tile's rays in shared memory
 * and flushes it with float4 atomics; 1 = one global atomic per tap (the
 * same sums in another order).  One key changes results: the
 * precision form, "flow_bits" = 16 stores the flow solver's dual, flow and
 * linearisation as FP16 pairs during the primal-dual iterations and computes
 * them with fused multiply-adds and hardware reciprocals (FP64 residual sums;
 * grids with nx % 4 == 0, others stay FP32), grows the flow pyramid in float
 * instead of double, and gives the flow solver's and warp-and-project's
 * warps a fused-multiply-add cubic; the standalone calls (wap_advect,
 * wap_resize, wap_blur) keep the reference's arithmetic.  32 (the default) is
 * the reference's arithmetic everywhere.  Each precision keeps its own
 * autotuned plans.  Unknown keys are WAP_EINVAL. */
WAP_API int wap_set_tuning(wap_ctx *ctx, const char *key, int value);
/* The form and z-chunk used for a grid (after its first flow level; before
 * that, the forced values or 0). */
WAP_API int wap_get_tuning(wap_ctx *ctx, const int *dims, int *h_form, int *h_zchunk);

/* Projection stack W*H*nproj (PSART ctor loading + get_split, WaP_Tomo.cpp:339);
 * also sets G_Max = max of the first projection image, projslevel[0][0]
 * (WaP_Tomo.cpp:347-348). */
WAP_API int wap_upload_projections(wap_ctx *ctx, const float *h_projs);
WAP_API int wap_set_projections_device(wap_ctx *ctx, const float *d_projs);
WAP_API float wap_gmax(const wap_ctx *ctx);
WAP_API int wap_set_gmax(wap_ctx *ctx, float gmax);

/* Frame windows of a time level (VolumeData::ReadStructuredFile,
 * VolumeData.cpp:118-228).  Returns the frame count, fills up to cap entries. */
WAP_API int wap_level_frames(const wap_scan_desc *scan, int level, int *start, int *end, float *ftime, float *tunit,
                             int cap);

/* Device state of one time level: F volumes, F flows, CP state (zeroed).
 * Frames and flows are then read/written with the calls below. */
WAP_API int wap_level_setup(wap_ctx *ctx, int level);
WAP_API int wap_level_nframes(const wap_ctx *ctx);
WAP_API int wap_frame_volume_upload(wap_ctx *ctx, int frame, const float *h_vol);
WAP_API int wap_frame_volume_download(wap_ctx *ctx, int frame, float *h_vol);
WAP_API int wap_frame_flow_upload(wap_ctx *ctx, int frame, const float *h_flow);
WAP_API int wap_frame_flow_download(wap_ctx *ctx, int frame, float *h_flow);
WAP_API float *wap_frame_volume_device(wap_ctx *ctx, int frame);
WAP_API float *wap_frame_flow_device(wap_ctx *ctx, int frame);
/* Next time level: frame 2i and 2i+1 take frame i (WaP_Tomo.cpp:834-849). */
WAP_API int wap_level_advance(wap_ctx *ctx);

/* ---- projector (device pointers) ---------------------------------------- */

/* GenerateImage_GetCorrections (TypicalRayProducer.core.h:230-268) with
 * SingleScalarVolumePrepare/RayCasterPrepare (SingleScalarVolume.core.h:366,
 * RayCaster.core.h:191): projection d_img, ray length d_len and sample count
 * d_weight (W*H each; any may be NULL) of d_vol at projection `proj`. */
WAP_API int wap_forward_project(wap_ctx *ctx, int proj, const float *d_vol, float *d_img, float *d_len,
                                float *d_weight);

/* Batched form: njobs volumes, each at its own projection. */
WAP_API int wap_forward_project_batch(wap_ctx *ctx, int njobs, const int *h_proj, const float *const *h_d_vols,
                                      float *const *h_d_imgs, float *const *h_d_lens, float *const *h_d_weights);

/* PSART correction + dual update (WaP_Tomo.cpp:1530-1555): c = (p - Ax - y)/
 * (len + 1), y += alpha c.  d_dual may be NULL (y = 0, WaP_Tomo.cpp:1261-1284). */
WAP_API int wap_correction(wap_ctx *ctx, int n, const float *d_meas, const float *d_img, const float *d_len,
                           float *d_dual, float *d_corr);

/* Voxel-driven bicubic backprojection (WaP_Tomo.cpp:1557-1628 mode 0: vol +=
 * alpha*g then clamp [0,G_Max] over the box; WaP_Tomo.cpp:1294-1374 mode 1:
 * d_vol += g).  box = x0,x1,y0,y1,z0,z1 half-open; exact selects the
 * reference's double arithmetic. */
WAP_API int wap_backproject_voxel(wap_ctx *ctx, int proj, const float *d_corr, const int *box, int mode, int exact,
                                  float *d_vol);

/* Ray-driven matched backprojection: the reference's back-projection mode of
 * the ray caster (SingleScalarVolume.core.h:85-96,149-199): every sample of
 * the forward projector's march adds corr * w_k and w_k to its 8 trilinear
 * taps.  Accumulated in shared memory per slab of a tile's rays, flushed with
 * FP32 atomics (the sums' order varies from run to run).  d_contrib /
 * d_weight are accumulated into (zero them first). */
WAP_API int wap_backproject_ray(wap_ctx *ctx, int proj, const float *d_corr, float *d_contrib, float *d_weight);

/* ---- warp (device pointers) --------------------------------------------- */

/* advection::advect (advection.h:117-146): d_out (nc channels) = d_src warped
 * by the 3-channel d_vel over time dt inside the box aabb. */
WAP_API int wap_advect(wap_ctx *ctx, const int *dims, const float *aabb, const float *d_vel, const float *d_src,
                       int nc, float dt, float *d_out);

/* Self-check of the warp's arithmetic: CImg's cubic evaluated two lanes at a
 * time in packed FP32 instructions against the scalar evaluation, on n
 * pseudo-random input pairs drawn from seed (any float bits, subnormals,
 * signed zeros, dyadic values; fractions mostly in [0, 1)), in the reference
 * and the precision form's arithmetic.  *h_mismatches = the results whose
 * bits differ (0 expected; NaN against NaN counts as equal). */
WAP_API int wap_check_packed_cubic(wap_ctx *ctx, unsigned long long n, unsigned long long seed,
                                   unsigned long long *h_mismatches);

/* ---- optical flow (device pointers) ------------------------------------- */

/* CImg get_blur(sigma) (Deriche, CImg.h:33276-33285), get_resize(..,5)
 * (CImg.h:28432-28610) and get_gradient("xyz",0) (CImg.h:34570-34590) as the
 * flow pyramid uses them. */
WAP_API int wap_blur(wap_ctx *ctx, const int *dims, int nc, float sigma, const float *d_src, float *d_out);
WAP_API int wap_resize(wap_ctx *ctx, const int *dims, int nc, const float *d_src, const int *odims, float *d_out);

/* optical_flow::L1TVOpticalFlowNonlinear3D (optical_flow.h:88-995): one
 * pyramid level.  d_V (3 ch), d_Y1..d_Y3 (3 ch), d_Y4 (1 ch) are updated in
 * place (ROI written, as the reference does).  roi6 = margins.  Returns the
 * primal-dual iteration count of each warp in h_iters (nwarps ints). */
WAP_API int wap_flow_level(wap_ctx *ctx, const int *dims, const float *d_I1, const float *d_I2, float *d_V,
                           float *d_Y1, float *d_Y2, float *d_Y3, float *d_Y4, float tol, float lambda,
                           int max_iters, int nwarps, const float *aabb, const int *roi6, int *h_iters);

/* optical_flow::L1TVOpticalFlowNonlinear_MultiScale3D (optical_flow.h:1002-1126)
 * as PSART::Render calls it (WaP_Tomo.cpp:711-753): Y start at zero, d_V0 is
 * the warm start, d_Vout the finest flow.  Returns total PD iterations via
 * h_total_iters (may be NULL). */
WAP_API int wap_flow_multiscale(wap_ctx *ctx, const int *dims, const float *d_I1, const float *d_I2,
                                const float *d_V0, float tol, float lambda, int max_iters, int nwarps, float eta,
                                float sigma, int scales, const int *cut6, float *d_Vout, long long *h_total_iters);

/* The same with the dual fields' warm start (the reference's Y1..Y4
 * arguments, resized to the coarsest level like V0; NULL for all four = zero,
 * which is what PSART::Render passes). */
WAP_API int wap_flow_multiscale_warm(wap_ctx *ctx, const int *dims, const float *d_I1, const float *d_I2,
                                     const float *d_V0, const float *d_Y1, const float *d_Y2, const float *d_Y3,
                                     const float *d_Y4, float tol, float lambda, int max_iters, int nwarps, float eta,
                                     float sigma, int scales, const int *cut6, float *d_Vout,
                                     long long *h_total_iters);

/* ---- solver (context state) -------------------------------------------- */

/* PSART::SART_Proximal_Operator (WaP_Tomo.cpp:1424-1678) on one frame of the
 * current level; use_cut selects the ROI box of Render (cut margins). */
WAP_API int wap_sart_prox(wap_ctx *ctx, int frame, int nb_sart, int cut, int exact);

/* PSART::WarpAndProjct (WaP_Tomo.cpp:1207-1421) for one projection. */
WAP_API int wap_warp_and_project(wap_ctx *ctx, int frame, int proj, float rtime, int exact);

/* PSART::AdaptiveWarp (WaP_Tomo.cpp:878-1204; commented out in the reference)
 * on one frame of the current level: nb_warp sweeps over the frame's window
 * in order, each projection forward-projecting the volume warped by
 * flow[max(0, frame-1)] (correction against one dual row, zeroed per call),
 * backprojecting into a delta volume that accumulates over the sweep (ROI box
 * from cut), and adding alpha * the delta warped back by flow[max(0, frame-2)]
 * then clamping to [0, G_Max]; max(vol, 0) at the end.  The reference's
 * per-projection time (m_ProjIndex[i].rElapsed) is never set; the warp-and-
 * project step's clamp((i - fTime) / tunit, -1, 1) is used. */
WAP_API int wap_adaptive_warp(wap_ctx *ctx, int frame, int nb_warp, int cut, int exact);

/* One outer iteration of PSART::Render at the current level
 * (WaP_Tomo.cpp:514-827): CP prior + SART over all frames, flow for every
 * adjacent pair, warp-and-project over the schedule's frames. */
WAP_API int wap_outer_iteration(wap_ctx *ctx, const wap_schedule *sched, wap_stats *stats);

/* The same outer iteration restricted to frames [f0, f1): their CP + SART
 * steps, the flows of the pairs (f, f+1) they start, and their WaP windows.
 * [0, F) is wap_outer_iteration; a single frame is one frame's share of the
 * iteration's work (the unit the throughput benchmark streams). */
WAP_API int wap_outer_iteration_frames(wap_ctx *ctx, const wap_schedule *sched, int f0, int f1, wap_stats *stats);

/* The outer iteration as an ordered list of steps, for callers that
 * interleave several reconstructions on one GPU: steps 0..n_cp-1 are the CP
 * iterations over all frames (dual, primal, SART, over-relaxation), the next
 * F-1 steps the flows of the pairs (f, f+1), the last the warp-and-project
 * pass.  Running the steps 0..nsteps-1 in order is exactly
 * wap_outer_iteration. */
WAP_API int wap_outer_iteration_nsteps(const wap_ctx *ctx, const wap_schedule *sched);
WAP_API int wap_outer_iteration_step(wap_ctx *ctx, const wap_schedule *sched, int step, wap_stats *stats);

/* Per-projection matrices as the projector kernels use them (host only, no
 * GPU needed): the reference's PixelsToModel, ModelToVolume, model-view x
 * VolumeToModel, and EyePos (TypicalRayProducer.cpp:157-232,
 * TypicalRayProducer.core.h:255-258). */
WAP_API int wap_projection_geometry(const wap_scan_desc *scan, double angle_deg, float *h_p2m, float *h_m2v,
                                    float *h_mvv2m, float *h_eye);

/* ---- CG (device pointers) ---------------------------------------------- */

/* image_cg::cg (cg.h:11-55) on A = a*I - b*Laplacian (Neumann): x updated in
 * place.  mode 0 is textbook CG; mode 1 reproduces the reference's update
 * (image_blas::add reassigns p before reading it, image_blas.h:135-149, so
 * p = r).  Dot products and norms in FP64, summed in a fixed order, so a
 * solve is reproducible bit for bit.  Returns iterations in h_iters (also on
 * failure).  An error left pending by the caller's earlier CUDA work is
 * reported as WAP_ECUDA before anything runs, and left pending. */
WAP_API int wap_cg_screened_laplacian(wap_ctx *ctx, const int *dims, float a, float b, const float *d_rhs,
                                      float *d_x, float rel_tol, int max_iters, float abs_tol, int mode,
                                      int *h_iters);

/* Allocation-free variant of wap_cg_screened_laplacian.  This entry point has
 * no counterpart in the reference.  It exists for callers that cannot have the
 * library allocate device memory: applications whose memory pool has reserved
 * the device, where an extra cudaMalloc fails, and serving loops that cannot
 * absorb the device-wide synchronisation of cudaFree.  Its scratch (the CG
 * vectors r, p, Ap, the FP64 per-block partial sums and four scalars) lives in
 * one fixed device array of 3 * WAP_CG_NOALLOC_MAX_VOXELS floats (3 MiB) plus
 * 16 KiB, which every GPU that loads the library holds until the process
 * exits.  Grids with more than
 * WAP_CG_NOALLOC_MAX_VOXELS voxels return WAP_ETOOBIG.  It needs no context:
 * it works on the current device and orders its work on cuda_stream (NULL =
 * the legacy default stream), with the same arguments and results as
 * wap_cg_screened_laplacian (bit for bit: both reduce in a fixed order).  The
 * first call on each device looks the scratch
 * address up (cudaGetSymbolAddress) with that device current; make that first
 * call before any stream capture.  Every call reuses the same scratch, so
 * calls that overlap on the GPU (other streams, other host threads) race. */
#define WAP_CG_NOALLOC_MAX_VOXELS 262144
WAP_API int wap_cg_screened_laplacian_noalloc(void *cuda_stream, const int *dims, float a, float b,
                                              const float *d_rhs, float *d_x, float rel_tol, int max_iters,
                                              float abs_tol, int mode, int *h_iters);

#ifdef __cplusplus
}
#endif
#endif /* WAP_WAP_H */
