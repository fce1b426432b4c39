"""ctypes binding of the C ABI in include/wap/wap.h (libwap_gb300.so).

This is the host-side view a Python caller (the tests, bench.py) uses.  Device
arrays are passed as raw pointers; torch CUDA tensors are accepted for
convenience (torch is only used for device memory here).  The library is
required: there is no CPU fallback, and loading fails loudly when the shared
object is missing.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libwap_gb300.so")

WAP_OK, WAP_EINVAL, WAP_ENOMEM, WAP_ECUDA, WAP_ESTATE, WAP_ENODEV, WAP_ETOOBIG, WAP_EIO, WAP_EHOST = range(9)

_c_int, _c_float, _c_double, _vp = ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_void_p


class ScanDesc(ctypes.Structure):
    _fields_ = [
        ("vol", _c_int * 3),
        ("det", _c_int * 2),
        ("nproj", _c_int),
        ("nframes_cli", _c_int),
        ("vs", _c_double),
        ("ds", _c_double),
        ("sid", _c_double),
        ("sdd", _c_double),
        ("oxyz", _c_double * 3),
        ("alpha", _c_double),
        ("tv_w", _c_double),
        ("tp_w", _c_double),
    ]


class Schedule(ctypes.Structure):
    _fields_ = [
        ("n_cp", _c_int),
        ("nb_sart", _c_int),
        ("nb_projwarp", _c_int),
        ("wp_frames", _c_int),
        ("flow_tol", _c_float),
        ("flow_lambda", _c_float),
        ("flow_iters", _c_int),
        ("flow_warps", _c_int),
        ("flow_eta", _c_float),
        ("flow_sigma", _c_float),
        ("flow_scales", _c_int),
        ("cut", _c_int),
        ("bp_exact", _c_int),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("flow_pd_iterations", ctypes.c_longlong),
        ("fp_launches", ctypes.c_longlong),
        ("kernel_launches", ctypes.c_longlong),
        ("ms_cp", _c_double),
        ("ms_flow", _c_double),
        ("ms_wap", _c_double),
        ("pd_voxel_iters", _c_double),
        ("advect_voxels", _c_double),
        ("projections", ctypes.c_longlong),
        ("backprojections", ctypes.c_longlong),
        ("cp_frame_passes", ctypes.c_longlong),
        ("ms_pd", _c_double),
        ("pd_timed", ctypes.c_longlong),
        ("pd_timed_voxels", ctypes.c_longlong),
        ("ms_flow_level", _c_double * 8),
        ("pd_iters_level", ctypes.c_longlong * 8),
    ]


class JobDesc(ctypes.Structure):
    _fields_ = [("scan", ScanDesc), ("sched", Schedule), ("outer_iterations", _c_int),
                ("h_angles", _vp), ("h_projs", _vp), ("flow_bits", _c_int)]


class JobInfo(ctypes.Structure):
    _fields_ = [("state", _c_int), ("status", _c_int), ("t_submit", _c_double), ("t_admit", _c_double),
                ("t_done", _c_double), ("steps", ctypes.c_longlong), ("device_bytes", ctypes.c_size_t)]


WAP_JOB_QUEUED, WAP_JOB_RUNNING, WAP_JOB_DONE, WAP_JOB_FAILED = range(4)

# wap_observer_fn: (user, event, level, a, b, d_data)
OBSERVER = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                            ctypes.c_void_p)
WAP_EV_SART, WAP_EV_FLOW, WAP_EV_WARP = 1, 2, 3

# Every function declared in include/wap/wap.h, with its ctypes signature.
SIGNATURES = {
    "wap_create_compute": (_c_int, [ctypes.POINTER(_vp), _c_int]),
    "wap_cached_bytes": (ctypes.c_size_t, []),
    "wap_trim_cache": (ctypes.c_size_t, [_c_int]),
    "wap_alloc": (_c_int, [_vp, ctypes.c_size_t, ctypes.POINTER(_vp)]),
    "wap_free": (_c_int, [_vp, _vp]),
    "wap_copy_to_device": (_c_int, [_vp, _vp, _vp, ctypes.c_size_t]),
    "wap_copy_to_host": (_c_int, [_vp, _vp, _vp, ctypes.c_size_t]),
    "wap_fill_zero": (_c_int, [_vp, _vp, ctypes.c_size_t]),
    "wap_set_observer": (_c_int, [_vp, OBSERVER, _vp]),
    "wap_create": (_c_int, [ctypes.POINTER(_vp), ctypes.POINTER(ScanDesc), _vp, _c_int]),
    "wap_destroy": (None, [_vp]),
    "wap_last_error": (ctypes.c_char_p, [_vp]),
    "wap_set_stream": (_c_int, [_vp, _vp]),
    "wap_synchronize": (_c_int, [_vp]),
    "wap_get_stats": (_c_int, [_vp, ctypes.POINTER(Stats)]),
    "wap_set_profiling": (_c_int, [_vp, _c_int]),
    "wap_set_tuning": (_c_int, [_vp, ctypes.c_char_p, _c_int]),
    "wap_get_tuning": (_c_int, [_vp, _vp, _vp, _vp]),
    "wap_upload_projections": (_c_int, [_vp, _vp]),
    "wap_set_projections_device": (_c_int, [_vp, _vp]),
    "wap_gmax": (_c_float, [_vp]),
    "wap_set_gmax": (_c_int, [_vp, _c_float]),
    "wap_level_frames": (_c_int, [ctypes.POINTER(ScanDesc), _c_int, _vp, _vp, _vp, _vp, _c_int]),
    "wap_level_setup": (_c_int, [_vp, _c_int]),
    "wap_level_nframes": (_c_int, [_vp]),
    "wap_frame_volume_upload": (_c_int, [_vp, _c_int, _vp]),
    "wap_frame_volume_download": (_c_int, [_vp, _c_int, _vp]),
    "wap_frame_flow_upload": (_c_int, [_vp, _c_int, _vp]),
    "wap_frame_flow_download": (_c_int, [_vp, _c_int, _vp]),
    "wap_frame_volume_device": (_vp, [_vp, _c_int]),
    "wap_frame_flow_device": (_vp, [_vp, _c_int]),
    "wap_level_advance": (_c_int, [_vp]),
    "wap_forward_project": (_c_int, [_vp, _c_int, _vp, _vp, _vp, _vp]),
    "wap_forward_project_batch": (_c_int, [_vp, _c_int, _vp, _vp, _vp, _vp, _vp]),
    "wap_correction": (_c_int, [_vp, _c_int, _vp, _vp, _vp, _vp, _vp]),
    "wap_backproject_voxel": (_c_int, [_vp, _c_int, _vp, _vp, _c_int, _c_int, _vp]),
    "wap_backproject_ray": (_c_int, [_vp, _c_int, _vp, _vp, _vp]),
    "wap_advect": (_c_int, [_vp, _vp, _vp, _vp, _vp, _c_int, _c_float, _vp]),
    "wap_blur": (_c_int, [_vp, _vp, _c_int, _c_float, _vp, _vp]),
    "wap_resize": (_c_int, [_vp, _vp, _c_int, _vp, _vp, _vp]),
    "wap_check_packed_cubic": (_c_int, [_vp, ctypes.c_ulonglong, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_ulonglong)]),
    "wap_flow_level": (_c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _c_float, _c_float, _c_int, _c_int,
                                _vp, _vp, _vp]),
    "wap_flow_multiscale": (_c_int, [_vp, _vp, _vp, _vp, _vp, _c_float, _c_float, _c_int, _c_int, _c_float,
                                     _c_float, _c_int, _vp, _vp, _vp]),
    "wap_flow_multiscale_warm": (_c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _c_float, _c_float, _c_int,
                                          _c_int, _c_float, _c_float, _c_int, _vp, _vp, _vp]),
    "wap_sart_prox": (_c_int, [_vp, _c_int, _c_int, _c_int, _c_int]),
    "wap_warp_and_project": (_c_int, [_vp, _c_int, _c_int, _c_float, _c_int]),
    "wap_adaptive_warp": (_c_int, [_vp, _c_int, _c_int, _c_int, _c_int]),
    "wap_outer_iteration": (_c_int, [_vp, ctypes.POINTER(Schedule), ctypes.POINTER(Stats)]),
    "wap_outer_iteration_frames": (_c_int, [_vp, ctypes.POINTER(Schedule), _c_int, _c_int, ctypes.POINTER(Stats)]),
    "wap_outer_iteration_nsteps": (_c_int, [_vp, ctypes.POINTER(Schedule)]),
    "wap_outer_iteration_step": (_c_int, [_vp, ctypes.POINTER(Schedule), _c_int, ctypes.POINTER(Stats)]),
    "wap_projection_geometry": (_c_int, [ctypes.POINTER(ScanDesc), _c_double, _vp, _vp, _vp, _vp]),
    "wap_cg_screened_laplacian": (_c_int, [_vp, _vp, _c_float, _c_float, _vp, _vp, _c_float, _c_int, _c_float,
                                           _c_int, _vp]),
    # include/wap/wap_serve.h
    "wap_job_device_bytes": (ctypes.c_size_t, [ctypes.POINTER(ScanDesc), ctypes.POINTER(Schedule)]),
    "wap_ctx_device_bytes": (ctypes.c_size_t, [_vp]),
    "wap_server_create": (_c_int, [ctypes.POINTER(_vp), _c_int, ctypes.c_size_t, _c_int]),
    "wap_server_destroy": (None, [_vp]),
    "wap_server_submit": (_c_int, [_vp, ctypes.POINTER(JobDesc), ctypes.POINTER(ctypes.c_longlong)]),
    "wap_server_info": (_c_int, [_vp, ctypes.c_longlong, ctypes.POINTER(JobInfo)]),
    "wap_server_wait": (_c_int, [_vp, ctypes.c_longlong, _c_double]),
    "wap_server_result": (_c_int, [_vp, ctypes.c_longlong, _c_int, _vp]),
    "wap_server_release": (_c_int, [_vp, ctypes.c_longlong]),
    "wap_server_now": (_c_double, [_vp]),
    "wap_server_memory": (_c_int, [_vp, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]),
    # include/wap/wap_io.h
    "wap_batch_create": (_c_int, [_vp, _vp, _c_int]),
    "wap_batch_destroy": (None, [_vp]),
    "wap_batch_last_error": (ctypes.c_char_p, [_vp]),
    "wap_batch_outer_iteration": (_c_int, [_vp, _vp, _vp]),
    "wap_batch_set_tuning": (_c_int, [_vp, _c_int, _c_int]),
    "wap_batch_get_tuning": (_c_int, [_vp, _vp, _vp]),
    "wap_tiff_info": (_c_int, [ctypes.c_char_p, _vp, _vp, _vp]),
    "wap_tiff_load": (_c_int, [ctypes.c_char_p, _vp, ctypes.c_size_t]),
    "wap_analyze_info": (_c_int, [ctypes.c_char_p, _vp, _vp]),
    "wap_analyze_load": (_c_int, [ctypes.c_char_p, _vp, ctypes.c_size_t]),
    "wap_analyze_save": (_c_int, [ctypes.c_char_p, _vp, _vp, _vp]),
    "wap_read_angles": (_c_int, [ctypes.c_char_p, _vp, _c_int, _vp]),
    "wap_split_z": (_c_int, [_c_int, _c_int, _vp, _vp]),
    "wap_lds_angles": (_c_int, [_c_int, _c_int, _c_int, _c_int, _vp]),
}

_lib = None


def load():
    """Load libwap_gb300.so (built by build.py); raise if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libwap_gb300.so is not built (run warp-and-project-tomography_gb300/build.py)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def ptr(x):
    """Raw pointer of a numpy array, a torch tensor, an int or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        assert x.flags["C_CONTIGUOUS"]
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        assert x.is_contiguous()
        return x.data_ptr()
    raise TypeError(type(x))


def _ints(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.int32))


def _floats(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float32))


class WapError(RuntimeError):
    pass


def make_scan(vol, det, nproj, nframes_cli=1, vs=1.0, ds=1.0, sid=None, sdd=None, oxyz=(0.0, 0.0, 0.0),
              alpha=0.1, tv_w=0.3, tp_w=0.3):
    n = vol[0]
    s = ScanDesc()
    s.vol[:] = list(vol)
    s.det[:] = list(det)
    s.nproj, s.nframes_cli = nproj, nframes_cli
    s.vs, s.ds = vs, ds
    s.sid = 4.0 * n if sid is None else sid
    s.sdd = 6.0 * n if sdd is None else sdd
    s.oxyz[:] = list(oxyz)
    s.alpha, s.tv_w, s.tp_w = alpha, tv_w, tp_w
    return s


def reference_schedule(n_cp=5, nb_sart=2, wp_frames=1, flow_iters=3000, flow_scales=5, flow_tol=0.008, cut=8,
                       bp_exact=1, flow_warps=3):
    """The constants PSART::Render hard-codes (WaP_Tomo.cpp:478-492, 711-727)."""
    return Schedule(n_cp=n_cp, nb_sart=nb_sart, nb_projwarp=1, wp_frames=wp_frames, flow_tol=flow_tol,
                    flow_lambda=0.05, flow_iters=flow_iters, flow_warps=flow_warps, flow_eta=0.5, flow_sigma=0.8,
                    flow_scales=flow_scales, cut=cut, bp_exact=bp_exact)


class Context:
    """One wap_ctx: a scan's geometry, projections and device frame state."""

    def __init__(self, scan, angles_deg, device=0):
        self.L = load()
        self.scan = scan
        self._observer = None
        h = _vp()
        if scan is None:  # compute-only context (wap_create_compute)
            self.angles = None
            r = self.L.wap_create_compute(ctypes.byref(h), device)
        else:
            self.angles = np.ascontiguousarray(np.asarray(angles_deg, np.float64))
            r = self.L.wap_create(ctypes.byref(h), ctypes.byref(scan), self.angles.ctypes.data, device)
        if r != WAP_OK:
            raise WapError("wap_create failed with status %d" % r)
        self.h = h

    @classmethod
    def compute(cls, device=0):
        """A context without a scan, for the grid-argument calls."""
        return cls(None, None, device)

    def set_observer(self, fn):
        """fn(event, level, a, b, d_data_ptr) or None."""
        if fn is None:
            self._observer = None
            self.call("wap_set_observer", OBSERVER(), None)
            return
        self._observer = OBSERVER(lambda user, ev, lvl, a, b, d: fn(ev, lvl, a, b, d))
        self.call("wap_set_observer", self._observer, None)

    def copy_to_host(self, d_ptr, nfloats):
        out = np.empty(nfloats, np.float32)
        self.call("wap_copy_to_host", out.ctypes.data, d_ptr, out.nbytes)
        return out

    def close(self):
        if getattr(self, "h", None):
            self.L.wap_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, r, what):
        if r != WAP_OK:
            msg = self.L.wap_last_error(self.h)
            raise WapError("%s failed (%d): %s" % (what, r, msg.decode() if msg else ""))

    def call(self, name, *args):
        self._ok(getattr(self.L, name)(self.h, *args), name)

    # ---- state
    def upload_projections(self, projs):
        projs = np.ascontiguousarray(projs, np.float32)
        self.call("wap_upload_projections", projs.ctypes.data)

    def set_projections_device(self, dprojs):
        self.call("wap_set_projections_device", ptr(dprojs))

    @property
    def gmax(self):
        return self.L.wap_gmax(self.h)

    def set_gmax(self, g):
        self.call("wap_set_gmax", g)

    def level_setup(self, level):
        self.call("wap_level_setup", level)
        return self.L.wap_level_nframes(self.h)

    def level_advance(self):
        self.call("wap_level_advance")

    def upload_volume(self, f, vol):
        vol = np.ascontiguousarray(vol, np.float32)
        self.call("wap_frame_volume_upload", f, vol.ctypes.data)

    def download_volume(self, f):
        n = self.scan.vol
        out = np.zeros((n[2], n[1], n[0]), np.float32)
        self.call("wap_frame_volume_download", f, out.ctypes.data)
        return out

    def upload_flow(self, f, flow):
        flow = np.ascontiguousarray(flow, np.float32)
        self.call("wap_frame_flow_upload", f, flow.ctypes.data)

    def download_flow(self, f):
        n = self.scan.vol
        out = np.zeros((3, n[2], n[1], n[0]), np.float32)
        self.call("wap_frame_flow_download", f, out.ctypes.data)
        return out

    def volume_device(self, f):
        return self.L.wap_frame_volume_device(self.h, f)

    def flow_device(self, f):
        return self.L.wap_frame_flow_device(self.h, f)

    def set_profiling(self, on):
        self.call("wap_set_profiling", 1 if on else 0)

    def set_tuning(self, key, value):
        self.call("wap_set_tuning", key.encode(), int(value))

    def get_tuning(self, dims):
        d = _ints(dims)
        f, z = ctypes.c_int(0), ctypes.c_int(0)
        self.call("wap_get_tuning", d.ctypes.data, ctypes.addressof(f), ctypes.addressof(z))
        return f.value, z.value

    def set_stream(self, stream_ptr):
        self.call("wap_set_stream", stream_ptr)

    def synchronize(self):
        self.call("wap_synchronize")

    def stats(self):
        s = Stats()
        self.call("wap_get_stats", ctypes.byref(s))
        return s

    # ---- kernels on device pointers
    def forward(self, proj, d_vol, d_img, d_len=None, d_weight=None):
        self.call("wap_forward_project", proj, ptr(d_vol), ptr(d_img), ptr(d_len), ptr(d_weight))

    def correction(self, n, d_meas, d_img, d_len, d_dual, d_corr):
        self.call("wap_correction", n, ptr(d_meas), ptr(d_img), ptr(d_len), ptr(d_dual), ptr(d_corr))

    def backproject_voxel(self, proj, d_corr, box, mode, exact, d_vol):
        b = _ints(box)
        self.call("wap_backproject_voxel", proj, ptr(d_corr), b.ctypes.data, mode, exact, ptr(d_vol))

    def backproject_ray(self, proj, d_corr, d_contrib, d_weight):
        self.call("wap_backproject_ray", proj, ptr(d_corr), ptr(d_contrib), ptr(d_weight))

    def advect(self, dims, aabb, d_vel, d_src, nc, dt, d_out):
        d, a = _ints(dims), _floats(aabb)
        self.call("wap_advect", d.ctypes.data, a.ctypes.data, ptr(d_vel), ptr(d_src), nc, dt, ptr(d_out))

    def blur(self, dims, nc, sigma, d_src, d_out):
        d = _ints(dims)
        self.call("wap_blur", d.ctypes.data, nc, sigma, ptr(d_src), ptr(d_out))

    def resize(self, dims, nc, d_src, odims, d_out):
        d, o = _ints(dims), _ints(odims)
        self.call("wap_resize", d.ctypes.data, nc, ptr(d_src), o.ctypes.data, ptr(d_out))

    def check_packed_cubic(self, n, seed=0):
        """Bit mismatches between the warp's packed-pair cubic and the scalar
        one on n pseudo-random input pairs (0 expected)."""
        bad = ctypes.c_ulonglong(0)
        self.call("wap_check_packed_cubic", n, seed, ctypes.byref(bad))
        return bad.value

    def flow_level(self, dims, dI1, dI2, dV, dY1, dY2, dY3, dY4, tol, lam, iters, nwarps, aabb, roi6):
        d, a, r = _ints(dims), _floats(aabb), _ints(roi6)
        its = np.zeros(max(nwarps, 1), np.int32)
        self.call("wap_flow_level", d.ctypes.data, ptr(dI1), ptr(dI2), ptr(dV), ptr(dY1), ptr(dY2), ptr(dY3),
                  ptr(dY4), tol, lam, iters, nwarps, a.ctypes.data, r.ctypes.data, its.ctypes.data)
        return its

    def flow_multiscale(self, dims, dI1, dI2, dV0, tol, lam, iters, nwarps, eta, sigma, scales, cut6, dVout):
        d, c = _ints(dims), _ints(cut6)
        tot = ctypes.c_longlong(0)
        self.call("wap_flow_multiscale", d.ctypes.data, ptr(dI1), ptr(dI2), ptr(dV0), tol, lam, iters, nwarps, eta,
                  sigma, scales, c.ctypes.data, ptr(dVout), ctypes.addressof(tot))
        return tot.value

    def sart_prox(self, frame, nb_sart=2, cut=8, exact=1):
        self.call("wap_sart_prox", frame, nb_sart, cut, exact)

    def warp_and_project(self, frame, proj, rtime, exact=1):
        self.call("wap_warp_and_project", frame, proj, rtime, exact)

    def adaptive_warp(self, frame, nb_warp=1, cut=8, exact=1):
        self.call("wap_adaptive_warp", frame, nb_warp, cut, exact)

    def outer_iteration(self, sched):
        st = Stats()
        self.call("wap_outer_iteration", ctypes.byref(sched), ctypes.byref(st))
        return st

    def outer_iteration_frames(self, sched, f0, f1):
        st = Stats()
        self.call("wap_outer_iteration_frames", ctypes.byref(sched), f0, f1, ctypes.byref(st))
        return st

    def outer_iteration_nsteps(self, sched):
        return self.L.wap_outer_iteration_nsteps(self.h, ctypes.byref(sched))

    def outer_iteration_step(self, sched, step):
        st = Stats()
        self.call("wap_outer_iteration_step", ctypes.byref(sched), int(step), ctypes.byref(st))
        return st

    def cg_screened_laplacian(self, dims, a, b, d_rhs, d_x, rel_tol=1e-6, max_iters=500, abs_tol=1e-9, mode=0):
        d = _ints(dims)
        it = _c_int(0)
        self.call("wap_cg_screened_laplacian", d.ctypes.data, a, b, ptr(d_rhs), ptr(d_x), rel_tol, max_iters,
                  abs_tol, mode, ctypes.addressof(it))
        return it.value


class Batch:
    """wap_batch (include/wap/wap_batch.h): scans of uneven sizes reconstructed
    together, their SART steps in work-queue launches, the CP iteration a CUDA
    graph, flows and warp-and-project overlapped on the scans' streams.  The
    contexts are borrowed and must stay open."""

    def __init__(self, contexts):
        self.L = load()
        self.contexts = list(contexts)
        arr = (_vp * len(self.contexts))(*[c.h for c in self.contexts])
        h = _vp()
        r = self.L.wap_batch_create(ctypes.byref(h), arr, len(self.contexts))
        if r != WAP_OK:
            raise WapError("wap_batch_create failed with status %d" % r)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.wap_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def outer_iteration(self, scheds):
        arr = (Schedule * len(scheds))(*scheds)
        st = Stats()
        r = self.L.wap_batch_outer_iteration(self.h, arr, ctypes.byref(st))
        if r != WAP_OK:
            msg = self.L.wap_batch_last_error(self.h)
            raise WapError("wap_batch_outer_iteration failed (%d): %s" % (r, msg.decode() if msg else ""))
        return st

    def set_tuning(self, fp_shape=-1, bp_shape=-1):
        if self.L.wap_batch_set_tuning(self.h, fp_shape, bp_shape) != WAP_OK:
            raise WapError("wap_batch_set_tuning failed")

    def get_tuning(self):
        a, b = _c_int(0), _c_int(0)
        self.L.wap_batch_get_tuning(self.h, ctypes.addressof(a), ctypes.addressof(b))
        return a.value, b.value


def projection_geometry(scan, angle_deg):
    """Host-only: the projector's per-projection matrices (no GPU needed)."""
    L = load()
    out = [np.zeros(16, np.float32) for _ in range(3)] + [np.zeros(4, np.float32)]
    r = L.wap_projection_geometry(ctypes.byref(scan), angle_deg, *[o.ctypes.data for o in out])
    if r != WAP_OK:
        raise WapError("wap_projection_geometry failed (%d)" % r)
    return out


def level_frames(scan, level):
    L = load()
    st = np.zeros(130, np.int32)
    en = np.zeros(130, np.int32)
    ft = np.zeros(130, np.float32)
    tu = _c_float()
    nf = L.wap_level_frames(ctypes.byref(scan), level, st.ctypes.data, en.ctypes.data, ft.ctypes.data,
                            ctypes.addressof(tu), 130)
    return nf, st[:nf].copy(), en[:nf].copy(), ft[:nf].copy(), tu.value


# ---- host formats (include/wap/wap_io.h) -----------------------------------

def _path(p):
    return os.fsencode(p)


def tiff_info(path):
    """(W, H, pages, samples per pixel), bits, sample format of a TIFF stack."""
    d = np.zeros(4, np.int32)
    b, f = ctypes.c_int(0), ctypes.c_int(0)
    r = load().wap_tiff_info(_path(path), d.ctypes.data, ctypes.addressof(b), ctypes.addressof(f))
    if r != WAP_OK:
        raise WapError("wap_tiff_info(%s) failed with status %d" % (path, r))
    return tuple(int(x) for x in d), b.value, f.value


def tiff_load(path):
    """A TIFF stack as float32 (pages, H, W), as CImg<float>::load_tiff reads it."""
    (w, h, p, c), _, _ = tiff_info(path)
    out = np.zeros((p, h, w), np.float32)
    r = load().wap_tiff_load(_path(path), out.ctypes.data, out.size)
    if r != WAP_OK:
        raise WapError("wap_tiff_load(%s) failed with status %d" % (path, r))
    return out


def analyze_info(path):
    """(W, H, D, C), Analyze datatype code."""
    d = np.zeros(4, np.int32)
    t = ctypes.c_int(0)
    r = load().wap_analyze_info(_path(path), d.ctypes.data, ctypes.addressof(t))
    if r != WAP_OK:
        raise WapError("wap_analyze_info(%s) failed with status %d" % (path, r))
    return tuple(int(v) for v in d), t.value


def analyze_load(path):
    """Float array of shape (C, D, H, W) (CImg order: x fastest)."""
    (w, h, d, c), _ = analyze_info(path)
    out = np.empty((c, d, h, w), np.float32)
    r = load().wap_analyze_load(_path(path), out.ctypes.data, out.size)
    if r != WAP_OK:
        raise WapError("wap_analyze_load(%s) failed with status %d" % (path, r))
    return out


def analyze_save(path, arr, voxel_size=None):
    """arr: (W,) .. (C, D, H, W) float array, CImg order."""
    a = np.ascontiguousarray(arr, np.float32)
    shp = list(a.shape[::-1]) + [1] * (4 - a.ndim)
    dims = _ints(shp[:4])
    vs = None if voxel_size is None else _floats(voxel_size)
    r = load().wap_analyze_save(_path(path), a.ctypes.data, dims.ctypes.data, None if vs is None else vs.ctypes.data)
    if r != WAP_OK:
        raise WapError("wap_analyze_save(%s) failed with status %d" % (path, r))


def read_angles(path, n):
    out = np.zeros(n, np.float64)
    got = ctypes.c_int(0)
    r = load().wap_read_angles(_path(path), out.ctypes.data, n, ctypes.addressof(got))
    if r != WAP_OK:
        raise WapError("wap_read_angles(%s) failed with status %d" % (path, r))
    return out, got.value


def split_z(depth, nb):
    first = np.zeros(nb, np.int32)
    count = np.zeros(nb, np.int32)
    r = load().wap_split_z(depth, nb, first.ctypes.data, count.ctypes.data)
    if r != WAP_OK:
        raise WapError("wap_split_z(%d, %d) failed with status %d" % (depth, nb, r))
    return first, count


def lds_angles(np_, ns=1, p=2, nz=50):
    out = np.zeros(np_, np.float64)
    r = load().wap_lds_angles(np_, ns, p, nz, out.ctypes.data)
    if r != WAP_OK:
        raise WapError("wap_lds_angles failed with status %d" % r)
    return out


# ---- request loop (include/wap/wap_serve.h) ----------------------------------

def job_device_bytes(scan, sched):
    return int(load().wap_job_device_bytes(ctypes.byref(scan), ctypes.byref(sched)))


class Server:
    """Many reconstructions on one GPU, admitted by device footprint."""

    def __init__(self, budget_bytes, workers=2, device=0):
        self.L = load()
        h = _vp()
        r = self.L.wap_server_create(ctypes.byref(h), device, int(budget_bytes), int(workers))
        if r != WAP_OK:
            raise WapError("wap_server_create failed with status %d" % r)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.wap_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, scan, sched, angles, projs, outer_iterations=1, flow_bits=32):
        a = np.ascontiguousarray(angles, np.float64)
        p = np.ascontiguousarray(projs, np.float32)
        d = JobDesc(scan=scan, sched=sched, outer_iterations=int(outer_iterations), h_angles=a.ctypes.data,
                    h_projs=p.ctypes.data, flow_bits=int(flow_bits))
        jid = ctypes.c_longlong(0)
        r = self.L.wap_server_submit(self.h, ctypes.byref(d), ctypes.byref(jid))
        if r != WAP_OK:
            raise WapError("wap_server_submit failed with status %d" % r)
        return jid.value

    def info(self, jid):
        i = JobInfo()
        r = self.L.wap_server_info(self.h, jid, ctypes.byref(i))
        if r != WAP_OK:
            raise WapError("wap_server_info failed with status %d" % r)
        return i

    def wait(self, jid, timeout=600.0):
        return self.L.wap_server_wait(self.h, jid, float(timeout))

    def result(self, jid, frame, vol_shape):
        out = np.empty(vol_shape, np.float32)
        r = self.L.wap_server_result(self.h, jid, frame, out.ctypes.data)
        if r != WAP_OK:
            raise WapError("wap_server_result failed with status %d" % r)
        return out

    def release(self, jid):
        return self.L.wap_server_release(self.h, jid)

    def now(self):
        return self.L.wap_server_now(self.h)

    def memory(self):
        a, b = ctypes.c_size_t(0), ctypes.c_size_t(0)
        self.L.wap_server_memory(self.h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value
