/* wap_serve.h -- many reconstructions on one GPU: a request loop that keeps
 * each job's volumes, flows and projections resident on the device, admits
 * jobs by their device footprint against an HBM budget, interleaves their
 * outer-iteration steps (wap_outer_iteration_step) from several worker
 * threads on separate streams, and records per-job latency.
 *
 * The reference reconstructs one scan per process; this layer has no
 * counterpart there.  A job's result is the same alone and in the mix: its
 * steps run in order on its own context and no state is shared between jobs.
 */
#ifndef WAP_WAP_SERVE_H
#define WAP_WAP_SERVE_H

#include <stddef.h>

#include "wap/wap.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct wap_server wap_server;

typedef struct {
  wap_scan_desc scan;
  wap_schedule sched;
  int outer_iterations;   /* outer iterations at time level 0 */
  const double *h_angles; /* scan.nproj angles in degrees, copied at submit */
  const float *h_projs;   /* W*H*nproj projections, copied at submit */
  int flow_bits;          /* 0 or 32: the reference's arithmetic; 16: the precision form
                           * (wap_set_tuning "flow_bits") */
} wap_job_desc;

enum { WAP_JOB_QUEUED = 0, WAP_JOB_RUNNING = 1, WAP_JOB_DONE = 2, WAP_JOB_FAILED = 3 };

typedef struct {
  int state;            /* WAP_JOB_* */
  int status;           /* WAP_OK, or the status of the call that failed */
  double t_submit;      /* seconds on the server's clock (wap_server_now) */
  double t_admit;       /* admitted: device memory reserved, context made */
  double t_done;        /* results on the host */
  long long steps;      /* outer-iteration steps run */
  size_t device_bytes;  /* the footprint reserved at admission */
} wap_job_info;

/* Device bytes a job of this scan and schedule holds at its peak (frame
 * arenas, CP state, projection stack, flow workspaces of every pyramid
 * level, scratch): the admission footprint. */
WAP_API size_t wap_job_device_bytes(const wap_scan_desc *scan, const wap_schedule *sched);

/* Device bytes a context has asked for and holds now (a block reused from the
 * process's cache of freed blocks may be up to 1/8 larger than asked). */
WAP_API size_t wap_ctx_device_bytes(const wap_ctx *ctx);

/* workers: host threads stepping jobs (each job is stepped by one thread at
 * a time; different jobs run concurrently on their own streams). */
WAP_API int wap_server_create(wap_server **out, int device, size_t hbm_budget_bytes, int workers);
/* Stops the workers after their current steps; queued and running jobs are
 * dropped. */
WAP_API void wap_server_destroy(wap_server *s);
/* Queues a job (inputs copied); *h_id receives its id.  A job whose
 * footprint exceeds the whole budget is WAP_ETOOBIG. */
WAP_API int wap_server_submit(wap_server *s, const wap_job_desc *job, long long *h_id);
WAP_API int wap_server_info(wap_server *s, long long id, wap_job_info *out);
/* Blocks until the job is done or failed (WAP_OK / its failure status), or
 * timeout_s passes (WAP_ESTATE). */
WAP_API int wap_server_wait(wap_server *s, long long id, double timeout_s);
/* Frame volume of a finished job (W*H*D floats). */
WAP_API int wap_server_result(wap_server *s, long long id, int frame, float *h_vol);
/* Frees a finished job's results. */
WAP_API int wap_server_release(wap_server *s, long long id);
/* Seconds since the server was created. */
WAP_API double wap_server_now(const wap_server *s);
/* Device bytes reserved by admitted jobs now, and the peak so far. */
WAP_API int wap_server_memory(const wap_server *s, size_t *h_in_use, size_t *h_peak);

#ifdef __cplusplus
}
#endif
#endif /* WAP_WAP_SERVE_H */
