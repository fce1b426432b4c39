/* CPU oracle for the warp-and-project hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain C++/OpenMP restatement of the reference's CPU algorithm, used as
 * the checker by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py.  It is never linked into, called by, or substituted for the GPU
 * product.  Every function cites the reference file:line it restates; the
 * restatement is pinned bit-for-bit against the reference's own sources
 * (oracle/_ref, built by `make ref`) and against tests/golden fixtures.
 *
 * Layouts follow CImg: idx = x + W*(y + H*z), channels planar.
 */
#ifndef WAP_ORACLE_H
#define WAP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* The oracle's arithmetic type: float (the restatement of the reference,
 * bit for bit) or, built with -DORC_REAL=double, double (the FP64 oracle:
 * the same algorithm with every float quantity in double). */
#ifndef ORC_REAL
#define ORC_REAL float
#endif
typedef ORC_REAL orc_real;


/* Scan + solver constants, as the reference's CLI sets them (main.cpp:15-138,
 * WaP_Tomo.cpp:228-434). */
typedef struct {
  int vol[3];       /* -f: volume dims */
  int det[2];       /* -u: detector W, H */
  int nproj;        /* total projections (main.cpp:198) */
  int nframes_cli;  /* -v: frames at time level 0 */
  double vs;        /* -c: voxel spacing */
  double ds;        /* -d: detector spacing */
  double sid;       /* -g: source to iso-centre */
  double sdd;       /* -j: source to detector */
  double oxyz[3];   /* --oxyz */
  double alpha;     /* -a: SART relaxation */
  double tv_w;      /* -s: TV weight */
  double tp_w;      /* -t: temporal weight */
  float gmax;       /* G_Max: max of the first projection image (WaP_Tomo.cpp:347-348) */
  int threads;      /* OpenMP threads, 0 = runtime default */
} orc_scan;

/* The schedule of one outer iteration (constants WaP_Tomo.cpp:478-492,711-727). */
typedef struct {
  int n_cp;           /* CP iterations (nb_volOpt[level]) */
  int nb_sart;        /* SART sweeps per proximal call (nb_proxiSART) */
  int nb_projwarp;    /* warp-and-project passes */
  int wp_frames;      /* frames the WaP pass visits (WaP_Tomo.cpp:801: CLI count) */
  float flow_tol;
  float flow_lambda;
  int flow_iters;
  int flow_warps;
  float flow_eta;
  float flow_sigma;
  int flow_scales;
  int cut;            /* ROI margin at full resolution (WaP_Tomo.cpp:114) */
  int deterministic;  /* 1: flow residual sums in loop order (single-thread reference) */
} orc_schedule;

/* Frame windows of one time level (VolumeData.cpp:133-210). */
int orc_level_frames(int nframes_cli, int nproj, int level, int *start, int *end, orc_real *ftime, orc_real *tunit);

/* Per-projection matrices (WaP_Tomo.cpp:1764-1797, Scene.cpp:65-189,
 * TypicalRayProducer.cpp:157-232, TypicalRayProducer.core.h:255-258). */
void orc_geometry(const orc_scan *s, double angle_deg, orc_real p2m[16], orc_real m2v[16], orc_real mv[16], orc_real v2m[16],
                  orc_real eye[4]);
orc_real orc_sample_distance(double vs);

/* Forward projector (TypicalRayProducer.core.h:32-225, RayCaster.core.h:42-188,
 * SingleScalarVolume.core.h:99-202).  img/len/weight: W*H. */
void orc_forward(const orc_scan *s, double angle_deg, const orc_real *vol, orc_real *img, orc_real *len, orc_real *weight);

/* The dead ray-driven backprojector (SingleScalarVolume.core.h:85-96,149-199). */
void orc_ray_backproject(const orc_scan *s, double angle_deg, const orc_real *corr, orc_real *contrib, orc_real *weight);

/* Correction + PSART dual (WaP_Tomo.cpp:1530-1555). */
void orc_correction(int n, const orc_real *p, const orc_real *ax, const orc_real *len, orc_real *dual, double alpha, orc_real *c);

/* Voxel-driven bicubic backprojection (WaP_Tomo.cpp:1557-1628 mode 0,
 * 1294-1374 mode 1).  box = x0,x1,y0,y1,z0,z1 (half-open). */
void orc_bp_voxel(const orc_scan *s, double angle_deg, const orc_real *corr, const int box[6], int mode, orc_real *vol);

/* advection::advect<orc_real> (advection.h:10-146, CImg.h:13429-13524). */
void orc_advect(const int dims[3], const orc_real aabb[6], const orc_real *vel, const orc_real *src, int nc, orc_real dt,
                orc_real *out, int threads);

/* CImg get_blur / get_resize(interp 5) / get_gradient("xyz",0). */
void orc_blur(const int dims[3], int nc, orc_real sigma, const orc_real *src, orc_real *out);
void orc_resize(const int dims[3], int nc, const orc_real *src, const int odims[3], orc_real *out);
void orc_gradient(const int dims[3], const orc_real *src, orc_real *gx, orc_real *gy, orc_real *gz);

/* One pyramid level of the L1-TV flow (optical_flow.h:88-995).  Returns the
 * total primal-dual iterations run; iters_out[w] gets each warp's count. */
int orc_flow_level(const int dims[3], const orc_real *I1, const orc_real *I2, orc_real *V, orc_real *Y1, orc_real *Y2, orc_real *Y3,
                   orc_real *Y4, orc_real tol, orc_real lambda, int max_iters, int nwarps, const orc_real aabb[6],
                   const int roi6[6], int deterministic, int *iters_out);

/* Wall time of the primal-dual loops of the last orc_flow_level call. */
double orc_last_pd_seconds(void);

/* Coarse-to-fine wrapper (optical_flow.h:1002-1126) as Render calls it. */
int orc_flow_multiscale(const int dims[3], const orc_real *I1, const orc_real *I2, const orc_real *V0, orc_real tol,
                        orc_real lambda, int max_iters, int nwarps, orc_real eta, orc_real sigma, int scales,
                        const int cut6[6], int deterministic, orc_real *Vout);

/* SART proximal operator on one frame (WaP_Tomo.cpp:1424-1678). */
void orc_sart_prox(const orc_scan *s, const double *angles, const orc_real *projs, int pstart, int pend, int nb_sart,
                   const int box[6], orc_real *vol, orc_real *dual_rows);
/* PSART::AdaptiveWarp (WaP_Tomo.cpp:878-1204, commented out in the reference)
 * on one frame: window [pstart, pend], frame time ftime, time unit tunit. */
void orc_adaptive_warp(const orc_scan *s, const double *angles, const orc_real *projs, int pstart, int pend,
                       orc_real ftime, orc_real tunit, int nb_warp, const int box[6], const orc_real *flow_fwd,
                       const orc_real *flow_adj, orc_real *vol);
/* The same with the ray-driven matched backprojection and column-sum
 * normalisation (--bp Raybased): vol += alpha * contrib / weight where
 * weight > 0, clamped to [0, G_Max], over the box. */
void orc_sart_prox_ray(const orc_scan *s, const double *angles, const orc_real *projs, int pstart, int pend,
                       int nb_sart, const int box[6], orc_real *vol, orc_real *dual_rows);

/* One warp-and-project step (WaP_Tomo.cpp:1207-1421). */
void orc_warp_and_project(const orc_scan *s, const double *angles, const orc_real *projs, int proj, orc_real rtime,
                          const orc_real *flow_fwd, const orc_real *flow_adj, orc_real *vol);

/* CP prior (WaP_Tomo.cpp:586-689), split the way the data flows:
 * dual of frame f, then primal of frame f before its SART call, then the
 * over-relaxation after it. */
void orc_cp_dual(const orc_scan *s, const int box[6], const orc_real *xbar_f, const orc_real *xbar_next, orc_real *ytv_f,
                 orc_real *ytp_f);
void orc_cp_primal(const orc_scan *s, const int box[6], int frame, const orc_real *ytp_prev, const orc_real *ytp_f,
                   const orc_real *ytv_f, orc_real *vol, orc_real *xprev);
void orc_cp_overrelax(const int dims[3], const int box[6], const orc_real *vol, const orc_real *xprev, orc_real *xbar);

/* Session over all frames of one time level: volumes F*V, flows F*3V and the
 * CP state; one call = one outer iteration (WaP_Tomo.cpp:514-827). */
int orc_outer_iteration(const orc_scan *s, const orc_schedule *sch, const double *angles, const orc_real *projs,
                        int level, orc_real *vols, orc_real *flows, orc_real *ytv, orc_real *ytp, orc_real *xbar, orc_real *xprev,
                        int *flow_iters_total);
/* The same restricted to frames [f0, f1): their CP + SART steps, the flows of
 * the pairs (f, f+1) they start and their warp-and-project windows. */
int orc_outer_iteration_frames(const orc_scan *s, const orc_schedule *sch, const double *angles, const orc_real *projs,
                               int level, int f0, int f1, orc_real *vols, orc_real *flows, orc_real *ytv,
                               orc_real *ytp, orc_real *xbar, orc_real *xprev, int *flow_iters_total);

/* image_cg::cg (cg.h:11-55) on A = a*I - b*Laplacian (clamped neighbours).
 * mode 0: textbook update p = r + beta*p; mode 1: the reference's aliasing
 * (image_blas.h:136-149 reassigns p before reading it -> p = r under zeroed
 * allocation).  Returns the iterations run. */
int orc_cg_screened_laplacian(const int dims[3], orc_real a, orc_real b, const orc_real *rhs, orc_real *x, orc_real rel_tol,
                              int max_iters, orc_real abs_tol, int mode);

#ifdef __cplusplus
}
#endif
#endif
