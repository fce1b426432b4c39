"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own sources (compiled headless by `make -C oracle ref`
into oracle/_ref/libwapref.so) on small seeded inputs and stores inputs and
outputs as .npz files.  Needs oracle/_ref/libwapref.so, built from the
reference tree by `make -C oracle ref REF=<tree>` (or by __graft_entry__.build()
where the tree is present); the tests only read the .npz files.
Single-threaded (OMP_NUM_THREADS=1) so the flow residual sums run in loop
order.

    OMP_NUM_THREADS=1 python tests/golden/make_golden.py
    python tests/golden/make_golden.py formats     # file formats only
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
sys.path.insert(0, os.path.join(HERE, ".."))
import oracle as O  # noqa: E402
import phantoms as P  # noqa: E402


def save(name, **arrays):
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    print("wrote", name, {k: v.shape for k, v in arrays.items()})


def projector_and_solver(ref, orc):
    N, W, H, NP = 24, 32, 32, 12
    vol = P.ellipsoids(N, count=8, seed=10)
    flow = P.rbf_flow(N, amp=1.5, seed=11)
    ang = P.golden_angles(NP)
    scan = O.make_scan((N, N, N), (W, H), NP, nframes_cli=2)
    projs = np.stack([orc.forward(scan, a, vol)[0] for a in ang]).astype(np.float32)
    projs += np.random.default_rng(12).normal(scale=0.01 * projs.max(), size=projs.shape).astype(np.float32)
    gmax = ref.create(scan, projs, ang, tempfile.mkdtemp())
    ref.lib.wref_set_volume(0, 0, vol)
    imgs, lens, wts = [], [], []
    for p in range(NP):
        i, l, w = (np.zeros((H, W), np.float32) for _ in range(3))
        ref.lib.wref_forward(0, 0, p, 0, 0.0, i, l, w)
        imgs.append(i)
        lens.append(l)
        wts.append(w)
    corr = np.random.default_rng(13).normal(size=(H, W)).astype(np.float32)
    rc = np.zeros((N, N, N), np.float32)
    rw = np.zeros_like(rc)
    ref.lib.wref_ray_backproject(0, 0, 3, corr, rc, rw)
    # SART proximal operator on frame 1, then warp-and-project on frame 1
    st, en, ft = O.ctypes.c_int(), O.ctypes.c_int(), O.ctypes.c_float()
    ref.lib.wref_frame_info(0, 1, O.ctypes.byref(st), O.ctypes.byref(en), O.ctypes.byref(ft))
    v1 = (vol * 0.5).astype(np.float32)
    ref.lib.wref_set_volume(0, 1, v1)
    ref.lib.wref_sart_prox(0, 1, 2, 1)
    sart = np.zeros_like(v1)
    ref.lib.wref_get_volume(0, 1, sart)
    fl0 = (flow * 0.7).astype(np.float32)
    ref.lib.wref_set_flow(0, 0, fl0)
    wap_steps = [(st.value, -0.6), (en.value, 0.9)]
    ref.lib.wref_warp_and_project(0, 1, wap_steps[0][0], wap_steps[0][1])
    ref.lib.wref_warp_and_project(0, 1, wap_steps[1][0], wap_steps[1][1])
    wap = np.zeros_like(v1)
    ref.lib.wref_get_volume(0, 1, wap)
    save("projector_solver", vol=vol, flow=flow, angles=ang, projs=projs, gmax=np.float32(gmax),
         img=np.stack(imgs), len=np.stack(lens), weight=np.stack(wts), corr=corr, raybp_contrib=rc, raybp_weight=rw,
         sart_in=v1, sart_window=np.array([st.value, en.value], np.int32), sart_out=sart, wap_flow0=fl0,
         wap_steps=np.array(wap_steps, np.float32), wap_out=wap, dims=np.array([N, N, W, H, NP], np.int32))
    ref.lib.wref_destroy()


def flow_components(ref, orc):
    N = 20
    dims = np.array([N, N, N], np.int32)
    aabb = np.array([0, N, 0, N, 0, N], np.float32)
    I1 = P.ellipsoids(N, count=6, seed=20)
    flow = P.rbf_flow(N, amp=1.5, seed=21)
    I2 = np.zeros_like(I1)
    ref.lib.wref_advect(dims, aabb, flow, I1, 1, 1.0, I2)
    adv = np.zeros_like(I1)
    ref.lib.wref_advect(dims, np.array([0, 2 * N, 0, 2 * N, 0, 2 * N], np.float32), flow, I1, 1, -0.7, adv)
    blur = np.zeros_like(I1)
    ref.lib.wref_blur(dims, 1, 0.8, I1, blur)
    down = np.zeros((3, 10, 10, 10), np.float32)
    ref.lib.wref_resize(dims, 3, flow, np.array([10, 10, 10], np.int32), down)
    up = np.zeros((3, 30, 27, 40), np.float32)
    ref.lib.wref_resize(dims, 3, flow, np.array([40, 27, 30], np.int32), up)
    g = [np.zeros_like(I1) for _ in range(3)]
    ref.lib.wref_gradient(dims, I1, *g)
    V = (flow * 0.3).astype(np.float32)
    Y = [np.zeros((3, N, N, N), np.float32) for _ in range(3)] + [np.zeros((N, N, N), np.float32)]
    roi = np.array([3] * 6, np.int32)
    ref.lib.wref_flow_level(dims, I1, I2, V, *Y, 0.0, 0.05, 40, 2, aabb, roi)
    Vm = np.zeros((3, N, N, N), np.float32)
    ref.lib.wref_flow_multiscale(dims, I1, I2, (flow * 0.5).astype(np.float32), 0.0, 0.05, 25, 2, 0.5, 0.8, 2,
                                 np.array([4] * 6, np.int32), Vm)
    rhs = np.random.default_rng(22).normal(size=(N, N, N)).astype(np.float32)
    x = np.zeros_like(rhs)
    ref.lib.wref_cg_screened_laplacian(dims, 1.0, 0.5, rhs, x, 1e-5, 60, 1e-9)
    save("flow_components", I1=I1, flow=flow, I2=I2, advect_box2=adv, blur=blur, resize_down=down, resize_up=up,
         gx=g[0], gy=g[1], gz=g[2], level_V=V, level_Y1=Y[0], level_Y2=Y[1], level_Y3=Y[2], level_Y4=Y[3],
         multiscale_V=Vm, cg_rhs=rhs, cg_x=x)


def render(ref, orc):
    """One complete PSART::Render (two time levels) at 48^3: the end-to-end pin."""
    N, W, H, NP = 48, 32, 32, 16
    vol = P.ellipsoids(N, count=10, seed=30)
    ang = P.golden_angles(NP)
    scan = O.make_scan((N, N, N), (W, H), NP, nframes_cli=1)
    projs = np.stack([orc.forward(scan, a, vol)[0] for a in ang]).astype(np.float32)
    gmax = ref.create(scan, projs, ang, tempfile.mkdtemp())
    r = ref.lib.wref_render()
    assert r == 0, r
    v0 = np.zeros((N, N, N), np.float32)
    v1 = np.zeros((N, N, N), np.float32)
    f0 = np.zeros((3, N, N, N), np.float32)
    ref.lib.wref_get_volume(1, 0, v0)
    ref.lib.wref_get_volume(1, 1, v1)
    ref.lib.wref_get_flow(1, 0, f0)
    save("render", projs=projs, angles=ang, gmax=np.float32(gmax), dims=np.array([N, N, W, H, NP], np.int32),
         level1_vol0=v0, level1_vol1=v1, level1_flow0=f0)
    ref.lib.wref_destroy()


def _analyze_header(dims4, datatype, bitpix, scale, vox_offset, big_endian, hsize=348):
    import struct
    e = ">" if big_endian else "<"
    h = bytearray(hsize)
    struct.pack_into(e + "i", h, 0, 348)
    struct.pack_into(e + "5h", h, 40, 4, *dims4)
    struct.pack_into(e + "h", h, 70, datatype)
    struct.pack_into(e + "h", h, 72, bitpix)
    struct.pack_into(e + "4f", h, 76, 0.0, 1.0, 1.0, 1.0)
    struct.pack_into(e + "f", h, 108, vox_offset)
    struct.pack_into(e + "f", h, 112, scale)
    return bytes(h)


def formats(ref):
    """Analyze/NIfTI files as CImg loads and saves them, and CImg's z-split."""
    rng = np.random.default_rng(40)
    dims4 = (5, 4, 3, 2)
    n = int(np.prod(dims4))
    cases = [  # name, numpy type, Analyze code, scale, big endian, single file
        ("f32_le", np.float32, 16, 0.5, False, False),
        ("i16_be", np.int16, 4, 0.0, True, False),
        ("u8_le", np.uint8, 2, 2.0, False, False),
        ("i32_le", np.int32, 8, 1.0, False, False),
        ("f64_nii", np.float64, 64, 1.0, False, True),
        ("f32_be_nii", np.float32, 16, 1.0, True, True),
    ]
    out = {}
    tmp = tempfile.mkdtemp()
    for name, dt, code, scale, be, single in cases:
        if np.issubdtype(dt, np.integer):
            info = np.iinfo(dt)
            data = rng.integers(max(info.min, -3000), min(info.max, 3000), size=n).astype(dt)
        else:
            data = (rng.normal(size=n) * 10).astype(dt)
        raw = data.astype(np.dtype(dt).newbyteorder(">" if be else "<")).tobytes()
        if single:
            hdr = _analyze_header(dims4, code, np.dtype(dt).itemsize, scale, 352.0, be, hsize=352)
            path = os.path.join(tmp, name + ".nii")
            open(path, "wb").write(hdr + raw)
        else:
            hdr = _analyze_header(dims4, code, np.dtype(dt).itemsize, scale, 0.0, be)
            path = os.path.join(tmp, name + ".hdr")
            open(path, "wb").write(hdr)
            open(os.path.join(tmp, name + ".img"), "wb").write(raw)
        got = np.zeros(n, np.float32)
        d = np.zeros(4, np.int32)
        assert ref.lib.wref_load_analyze(path.encode(), got, n, d) == 0, name
        assert tuple(d) == dims4
        out[name + "_hdr"] = np.frombuffer(hdr, np.uint8)
        out[name + "_raw"] = np.frombuffer(raw, np.uint8)
        out[name + "_loaded"] = got
    img = (rng.normal(size=dims4[::-1]) * 3).astype(np.float32)
    path = os.path.join(tmp, "saved.hdr")
    assert ref.lib.wref_save_analyze(path.encode(), img, np.array(dims4, np.int32)) == 0
    out["save_data"] = img
    out["save_hdr"] = np.frombuffer(open(path, "rb").read(), np.uint8)
    out["save_img"] = np.frombuffer(open(os.path.join(tmp, "saved.img"), "rb").read(), np.uint8)
    splits = [(192, 192), (200, 192), (7, 3), (10, 4), (33, 5), (5, 5), (9, 1), (384, 192), (191, 64)]
    table = []
    for depth, nb in splits:
        first = np.zeros(nb, np.int32)
        count = np.zeros(nb, np.int32)
        assert ref.lib.wref_split_z(depth, nb, first, count) == nb
        table.append(np.concatenate([[depth, nb], first, count]).astype(np.int32))
    out["split_table"] = np.concatenate(table)
    save("formats", **out)


if __name__ == "__main__":
    if sys.argv[1:] == ["formats"]:
        formats(O.Reference())
        sys.exit(0)
    if os.environ.get("OMP_NUM_THREADS") != "1":
        print("run with OMP_NUM_THREADS=1", file=sys.stderr)
        sys.exit(2)
    orc = O.Oracle()
    ref = O.Reference()
    projector_and_solver(ref, orc)
    flow_components(ref, orc)
    render(ref, orc)
