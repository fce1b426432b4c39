"""ctypes bindings for the CPU oracle (test infrastructure only).

Two libraries live under this directory:

* ``_build/libwaporacle.so`` -- the plain C++/OpenMP restatement of the
  reference's hot path (``wap_oracle.cpp``).  Buildable anywhere with g++.
  ``_build/libwaporacle64.so`` is the same source with every float quantity
  in double: the FP64 oracle (``Oracle(fp64=True)``, float64 arrays).
* ``_ref/libwapref.so`` -- the reference's own sources compiled headless with
  ``ref_harness.cpp`` (``make ref``).  Only buildable where the reference tree
  is present; used to pin the restatement and to generate tests/golden.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
import this module.  The GPU product never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libwaporacle.so")
ORACLE64_SO = os.path.join(HERE, "_build", "libwaporacle64.so")
REF_SO = os.path.join(HERE, "_ref", "libwapref.so")
REF_TREE_FILE = os.path.join(HERE, "_ref", "tree.txt")


def reference_tree():
    """The reference source tree: $WAP_REFERENCE_TREE, else the tree the last
    ``build_ref`` compiled (recorded in _ref/tree.txt), else None."""
    t = os.environ.get("WAP_REFERENCE_TREE")
    if not t and os.path.exists(REF_TREE_FILE):
        with open(REF_TREE_FILE) as f:
            t = f.read().strip()
    return t if t and os.path.isdir(os.path.join(t, "Project")) else None

_f32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64 = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_c_int, _c_float, _c_double = ctypes.c_int, ctypes.c_float, ctypes.c_double


class Scan(ctypes.Structure):
    """Mirror of ``orc_scan`` (wap_oracle.h)."""

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
        ("gmax", _c_float),
        ("threads", _c_int),
    ]


class Schedule(ctypes.Structure):
    """Mirror of ``orc_schedule`` (wap_oracle.h)."""

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
        ("deterministic", _c_int),
    ]


def make_scan(vol, det, nproj, nframes_cli=1, vs=1.0, ds=1.0, sid=None, sdd=None, oxyz=(0.0, 0.0, 0.0),
              alpha=0.1, tv_w=0.3, tp_w=0.3, gmax=1.0, threads=0):
    n = vol[0]
    s = Scan()
    s.vol[:] = list(vol)
    s.det[:] = list(det)
    s.nproj = nproj
    s.nframes_cli = nframes_cli
    s.vs, s.ds = vs, ds
    s.sid = 4.0 * n if sid is None else sid
    s.sdd = 6.0 * n if sdd is None else sdd
    s.oxyz[:] = list(oxyz)
    s.alpha, s.tv_w, s.tp_w = alpha, tv_w, tp_w
    s.gmax = gmax
    s.threads = threads
    return s


def build_oracle():
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)


def build_ref(tree=None):
    """Compile the reference's own sources found in ``tree`` (default:
    ``reference_tree()``) and record the tree for later calls."""
    tree = tree or reference_tree()
    if not tree or not os.path.isdir(os.path.join(tree, "Project")):
        return False
    subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", "REF=" + tree], check=True)
    with open(REF_TREE_FILE, "w") as f:
        f.write(os.path.abspath(tree) + "\n")
    return True


def _bind(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args
    return f


class Oracle:
    """The restatement (``wap_oracle.cpp``); fp64=True loads its FP64 build,
    whose arrays and scalars are float64."""

    def __init__(self, path=None, fp64=False):
        path = path or (ORACLE64_SO if fp64 else ORACLE_SO)
        if not os.path.exists(path):
            build_oracle()
        L = ctypes.CDLL(path)
        S = ctypes.POINTER(Scan)
        self.lib = L
        self.fp64 = fp64
        self.dt = np.float64 if fp64 else np.float32
        R = _f64 if fp64 else _f32  # arrays of the oracle's arithmetic type
        cR = _c_double if fp64 else _c_float  # its scalars
        _bind(L, "orc_level_frames", _c_int, [_c_int, _c_int, _c_int, _i32, _i32, R, ctypes.POINTER(cR)])
        _bind(L, "orc_geometry", None, [S, _c_double, R, R, R, R, R])
        _bind(L, "orc_sample_distance", cR, [_c_double])
        _bind(L, "orc_forward", None, [S, _c_double, R, R, R, R])
        _bind(L, "orc_ray_backproject", None, [S, _c_double, R, R, R])
        _bind(L, "orc_correction", None, [_c_int, R, R, R, ctypes.c_void_p, _c_double, R])
        _bind(L, "orc_bp_voxel", None, [S, _c_double, R, _i32, _c_int, R])
        _bind(L, "orc_advect", None, [_i32, R, R, R, _c_int, cR, R, _c_int])
        _bind(L, "orc_blur", None, [_i32, _c_int, cR, R, R])
        _bind(L, "orc_resize", None, [_i32, _c_int, R, _i32, R])
        _bind(L, "orc_gradient", None, [_i32, R, R, R, R])
        _bind(L, "orc_flow_level", _c_int, [_i32, R, R, R, R, R, R, R, cR, cR, _c_int, _c_int, R, _i32, _c_int,
                                            _i32])
        _bind(L, "orc_last_pd_seconds", _c_double, [])
        _bind(L, "orc_flow_multiscale", _c_int, [_i32, R, R, R, cR, cR, _c_int, _c_int, cR, cR, _c_int, _i32,
                                                 _c_int, R])
        _bind(L, "orc_sart_prox", None, [S, _f64, R, _c_int, _c_int, _c_int, _i32, R, R])
        _bind(L, "orc_sart_prox_ray", None, [S, _f64, R, _c_int, _c_int, _c_int, _i32, R, R])
        _bind(L, "orc_adaptive_warp", None, [S, _f64, R, _c_int, _c_int, cR, cR, _c_int, _i32, R, R, R])
        _bind(L, "orc_warp_and_project", None, [S, _f64, R, _c_int, cR, R, R, R])
        _bind(L, "orc_cp_dual", None, [S, _i32, R, R, R, R])
        _bind(L, "orc_cp_primal", None, [S, _i32, _c_int, ctypes.c_void_p, R, R, R, R])
        _bind(L, "orc_cp_overrelax", None, [_i32, _i32, R, R, R])
        _bind(L, "orc_outer_iteration", _c_int, [S, ctypes.POINTER(Schedule), _f64, R, _c_int, R, R, R, R, R, R,
                                                 ctypes.POINTER(_c_int)])
        _bind(L, "orc_outer_iteration_frames", _c_int, [S, ctypes.POINTER(Schedule), _f64, R, _c_int, _c_int,
                                                        _c_int, R, R, R, R, R, R, ctypes.POINTER(_c_int)])
        _bind(L, "orc_cg_screened_laplacian", _c_int, [_i32, cR, cR, R, R, cR, _c_int, cR, _c_int])

    def arr(self, x):
        """x as a contiguous array of the oracle's arithmetic type."""
        return np.ascontiguousarray(x, self.dt)

    # -- thin numpy wrappers ------------------------------------------------
    def level_frames(self, nframes_cli, nproj, level):
        st = np.zeros(130, np.int32)
        en = np.zeros(130, np.int32)
        ft = np.zeros(130, self.dt)
        tu = _c_double() if self.fp64 else _c_float()
        nf = self.lib.orc_level_frames(nframes_cli, nproj, level, st, en, ft, ctypes.byref(tu))
        return nf, st[:nf].copy(), en[:nf].copy(), ft[:nf].copy(), tu.value

    def geometry(self, scan, angle):
        out = [np.zeros(16, self.dt) for _ in range(4)] + [np.zeros(4, self.dt)]
        self.lib.orc_geometry(ctypes.byref(scan), angle, *out)
        return out

    def forward(self, scan, angle, vol):
        W, H = scan.det
        img, ln, wt = (np.zeros((H, W), self.dt) for _ in range(3))
        self.lib.orc_forward(ctypes.byref(scan), angle, self.arr(vol), img, ln, wt)
        return img, ln, wt

    def ray_backproject(self, scan, angle, corr):
        shp = tuple(reversed(list(scan.vol)))
        c = np.zeros(shp, self.dt)
        w = np.zeros(shp, self.dt)
        self.lib.orc_ray_backproject(ctypes.byref(scan), angle, self.arr(corr), c, w)
        return c, w

    def correction(self, p, ax, ln, dual, alpha):
        c = np.zeros_like(p, dtype=self.dt)
        dptr = dual.ctypes.data_as(ctypes.c_void_p) if dual is not None else None
        self.lib.orc_correction(p.size, p, ax, ln, dptr, alpha, c)
        return c

    def bp_voxel(self, scan, angle, corr, box, mode, vol):
        self.lib.orc_bp_voxel(ctypes.byref(scan), angle, corr, np.asarray(box, np.int32), mode, vol)
        return vol

    def advect(self, dims, aabb, vel, src, dt, threads=0):
        nc = src.size // int(np.prod(dims))
        out = np.zeros_like(src, dtype=self.dt)
        self.lib.orc_advect(np.asarray(dims, np.int32), self.arr(aabb), vel, src, nc, dt, out, threads)
        return out

    def blur(self, dims, src, sigma):
        nc = src.size // int(np.prod(dims))
        out = np.zeros_like(src, dtype=self.dt)
        self.lib.orc_blur(np.asarray(dims, np.int32), nc, sigma, src, out)
        return out

    def resize(self, dims, src, odims):
        nc = src.size // int(np.prod(dims))
        out = np.zeros((nc, odims[2], odims[1], odims[0]), self.dt)
        self.lib.orc_resize(np.asarray(dims, np.int32), nc, src, np.asarray(odims, np.int32), out)
        return out

    def gradient(self, dims, src):
        g = [np.zeros_like(src, dtype=self.dt) for _ in range(3)]
        self.lib.orc_gradient(np.asarray(dims, np.int32), src, *g)
        return g

    def flow_level(self, dims, I1, I2, V, Y1, Y2, Y3, Y4, tol, lam, iters, nwarps, aabb, roi, deterministic=1):
        its = np.zeros(max(nwarps, 1), np.int32)
        tot = self.lib.orc_flow_level(np.asarray(dims, np.int32), I1, I2, V, Y1, Y2, Y3, Y4, tol, lam, iters,
                                      nwarps, self.arr(aabb), np.asarray(roi, np.int32),
                                      deterministic, its)
        return tot, its

    def flow_multiscale(self, dims, I1, I2, V0, tol, lam, iters, nwarps, eta, sigma, scales, cut6,
                        deterministic=1):
        out = np.zeros_like(V0, dtype=self.dt)
        tot = self.lib.orc_flow_multiscale(np.asarray(dims, np.int32), I1, I2, V0, tol, lam, iters, nwarps, eta,
                                           sigma, scales, np.asarray(cut6, np.int32), deterministic, out)
        return out, tot

    def sart_prox(self, scan, angles, projs, pstart, pend, nb_sart, box, vol):
        W, H = scan.det
        dual = np.zeros((scan.nproj, H, W), self.dt)
        self.lib.orc_sart_prox(ctypes.byref(scan), angles, projs, pstart, pend, nb_sart, np.asarray(box, np.int32),
                               vol, dual)
        return vol, dual

    def sart_prox_ray(self, scan, angles, projs, pstart, pend, nb_sart, box, vol):
        W, H = scan.det
        dual = np.zeros((scan.nproj, H, W), self.dt)
        self.lib.orc_sart_prox_ray(ctypes.byref(scan), angles, projs, pstart, pend, nb_sart,
                                   np.asarray(box, np.int32), vol, dual)
        return vol, dual

    def adaptive_warp(self, scan, angles, projs, pstart, pend, ftime, tunit, nb_warp, box, flow_fwd, flow_adj, vol):
        self.lib.orc_adaptive_warp(ctypes.byref(scan), angles, projs, pstart, pend, ftime, tunit, nb_warp,
                                   np.asarray(box, np.int32), flow_fwd, flow_adj, vol)
        return vol

    def warp_and_project(self, scan, angles, projs, proj, rtime, flow_fwd, flow_adj, vol):
        self.lib.orc_warp_and_project(ctypes.byref(scan), angles, projs, proj, rtime, flow_fwd, flow_adj, vol)
        return vol

    def outer_iteration(self, scan, sched, angles, projs, level, state):
        tot = _c_int()
        F = self.lib.orc_outer_iteration(ctypes.byref(scan), ctypes.byref(sched), angles, projs, level,
                                         state["vols"], state["flows"], state["ytv"], state["ytp"], state["xbar"],
                                         state["xprev"], ctypes.byref(tot))
        return F, tot.value

    def outer_iteration_frames(self, scan, sched, angles, projs, level, f0, f1, state):
        tot = _c_int()
        F = self.lib.orc_outer_iteration_frames(ctypes.byref(scan), ctypes.byref(sched), angles, projs, level, f0,
                                                f1, state["vols"], state["flows"], state["ytv"], state["ytp"],
                                                state["xbar"], state["xprev"], ctypes.byref(tot))
        return F, tot.value

    def cg_screened_laplacian(self, dims, a, b, rhs, x, rel_tol=1e-6, max_iters=500, abs_tol=1e-9, mode=0):
        return self.lib.orc_cg_screened_laplacian(np.asarray(dims, np.int32), a, b, rhs, x, rel_tol, max_iters,
                                                  abs_tol, mode)


def lds_angles(np_, ns, p, nz):
    """Low-discrepancy scanning angles, a line-by-line restatement of
    Sampling_Model/low discrepancy sequence/Low_discrepency_squence.m:15-45
    (van der Corput radical inverse in base p over Ns circle segments, a
    0-degree projection before every Nz-th), in IEEE double like MATLAB."""
    seq = []
    i = 0
    while len(seq) < np_:
        if len(seq) > 0 and len(seq) % nz == 0:
            seq.append(0.0)
        b = i
        i += 1
        r = 0.0
        q = 1.0 / p
        while b != 0:
            a = b % p
            r = r + a * q
            q = q / p
            b = b // p
        r = 360 * r / ns
        k = 0
        while len(seq) < np_ and k < ns:
            seq.append(r + k * 360 / ns)
            k += 1
    return np.array(seq[:np_] if len(seq) > np_ else seq, np.float64)


class Reference:
    """The reference's own code (``_ref/libwapref.so``); one PSART session."""

    def __init__(self, path=REF_SO):
        if not os.path.exists(path):
            if not build_ref():
                raise RuntimeError("reference tree not available")
        L = ctypes.CDLL(path)
        self.lib = L
        _bind(L, "wref_create", _c_int, [_c_int] * 7 + [_c_double] * 7 + [_f64, _f32, _f64, ctypes.c_char_p])
        _bind(L, "wref_destroy", None, [])
        _bind(L, "wref_gmax", _c_float, [])
        _bind(L, "wref_level_info", _c_int, [_c_int, ctypes.POINTER(_c_int), ctypes.POINTER(_c_float)])
        _bind(L, "wref_frame_info", _c_int, [_c_int, _c_int, ctypes.POINTER(_c_int), ctypes.POINTER(_c_int),
                                             ctypes.POINTER(_c_float)])
        for nm in ("wref_set_volume", "wref_get_volume", "wref_set_flow", "wref_get_flow"):
            _bind(L, nm, _c_int, [_c_int, _c_int, _f32])
        _bind(L, "wref_geometry", _c_int, [_c_int, _f32, _f32, _f32, _f32, _f32])
        _bind(L, "wref_forward", _c_int, [_c_int, _c_int, _c_int, _c_int, _c_float, _f32, _f32, _f32])
        _bind(L, "wref_ray_backproject", _c_int, [_c_int, _c_int, _c_int, _f32, _f32, _f32])
        _bind(L, "wref_sart_prox", _c_int, [_c_int, _c_int, _c_int, _c_int])
        _bind(L, "wref_warp_and_project", _c_int, [_c_int, _c_int, _c_int, _c_float])
        _bind(L, "wref_render", _c_int, [])
        _bind(L, "wref_advect", _c_int, [_i32, _f32, _f32, _f32, _c_int, _c_float, _f32])
        _bind(L, "wref_blur", _c_int, [_i32, _c_int, _c_float, _f32, _f32])
        _bind(L, "wref_resize", _c_int, [_i32, _c_int, _f32, _i32, _f32])
        _bind(L, "wref_gradient", _c_int, [_i32, _f32, _f32, _f32, _f32])
        _bind(L, "wref_flow_level", _c_int, [_i32, _f32, _f32, _f32, _f32, _f32, _f32, _f32, _c_float, _c_float,
                                             _c_int, _c_int, _f32, _i32])
        _bind(L, "wref_flow_multiscale", _c_int, [_i32, _f32, _f32, _f32, _c_float, _c_float, _c_int, _c_int,
                                                  _c_float, _c_float, _c_int, _i32, _f32])
        _bind(L, "wref_cg_screened_laplacian", _c_int, [_i32, _c_float, _c_float, _f32, _f32, _c_float, _c_int,
                                                        _c_float])
        _bind(L, "wref_save_analyze", _c_int, [ctypes.c_char_p, _f32, _i32])
        _bind(L, "wref_load_analyze", _c_int, [ctypes.c_char_p, _f32, ctypes.c_longlong, _i32])
        _bind(L, "wref_split_z", _c_int, [_c_int, _c_int, _i32, _i32])

    def create(self, scan, projs, angles, workdir):
        r = self.lib.wref_create(scan.vol[0], scan.vol[1], scan.vol[2], scan.det[0], scan.det[1], scan.nproj,
                                 scan.nframes_cli, scan.vs, scan.ds, scan.sid, scan.sdd, scan.alpha, scan.tv_w,
                                 scan.tp_w, np.asarray(list(scan.oxyz), np.float64),
                                 np.ascontiguousarray(projs, np.float32), np.ascontiguousarray(angles, np.float64),
                                 workdir.encode())
        if r != 0:
            raise RuntimeError("wref_create failed")
        return self.lib.wref_gmax()
