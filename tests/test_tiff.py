"""TIFF projection stacks (CImg's libtiff loader, CImg.h:47445-47700, which the
reference enables for its projection input, WaP_Tomo.h:7-8): every page is
one z slice and each sample is cast to float.  Known-answer tests from the
TIFF 6.0 specification's PackBits and LZW examples, then stacks written here
in every layout the reader accepts (byte orders, strips and tiles, sample
types, compressions, the differencing predictor) read back exactly, and
malformed files refused.  No GPU needed."""
import struct
import zlib

import numpy as np
import pytest

TYPES = {np.uint8: (8, 1), np.int8: (8, 2), np.uint16: (16, 1), np.int16: (16, 2), np.uint32: (32, 1),
         np.int32: (32, 2), np.float32: (32, 3), np.float64: (64, 3)}


def packbits(data):
    """PackBits encoder (TIFF 6.0, section 9): literal runs of up to 128
    bytes, repeats of 2..128 bytes."""
    out, i, n = bytearray(), 0, len(data)
    while i < n:
        j = i
        while j + 1 < n and data[j + 1] == data[i] and j - i < 127:
            j += 1
        if j > i:
            out += bytes([(257 - (j - i + 1)) & 0xFF, data[i]])
            i = j + 1
            continue
        j = i
        while j < n and j - i < 128 and not (j + 1 < n and data[j + 1] == data[j]):
            j += 1
        j = max(j, i + 1)
        out += bytes([j - i - 1]) + data[i:j]
        i = j
    return bytes(out)


def lzw(data):
    """TIFF LZW encoder (TIFF 6.0, section 13): a Clear code first, 9-bit
    codes growing to 12 bits when the next free code passes 2^bits - 1, a
    Clear code when the table fills (4094 entries), the end code written at
    the width the decoder expects after the last data code."""
    codes = []
    width = 9

    def reset():
        return {bytes([i]): i for i in range(256)}, 258

    table, free = reset()
    codes.append((256, width))
    w = b""
    for c in data:
        wc = w + bytes([c])
        if wc in table:
            w = wc
            continue
        codes.append((table[w], width))
        table[wc] = free
        free += 1
        if free == 4094:
            codes.append((256, width))
            table, free = reset()
            width = 9
        elif free > (1 << width) - 1:
            width += 1
        w = bytes([c])
    if w:
        codes.append((table[w], width))
        free += 1
        if free == 4094:
            codes.append((256, width))
            width = 9
        elif free > (1 << width) - 1:
            width += 1
    codes.append((257, width))
    return pack_codes(codes)


def pack_codes(codes):
    acc, nbits, out = 0, 0, bytearray()
    for c, wdt in codes:
        acc = (acc << wdt) | c
        nbits += wdt
        while nbits >= 8:
            out.append((acc >> (nbits - 8)) & 0xFF)
            nbits -= 8
    if nbits:
        out.append((acc << (8 - nbits)) & 0xFF)
    return bytes(out)


def write_tiff(path, pages, order="<", comp=1, rps=None, tile=None, predictor=1, raw_blocks=None):
    """A multi-page TIFF of 2-D arrays (one sample per pixel)."""
    dt = pages[0].dtype
    bps, fmt = TYPES[dt.type]
    h, w = pages[0].shape
    out = bytearray(b"II*\x00" if order == "<" else b"MM\x00*")
    out += b"\x00\x00\x00\x00"
    link = 4  # where the previous IFD offset goes
    for z, img in enumerate(pages):
        a = img.astype(dt.newbyteorder(order))
        if tile:
            tw, th = tile
            blocks = []
            for by in range(0, h, th):
                for bx in range(0, w, tw):
                    t = np.zeros((th, tw), a.dtype)
                    sub = a[by:by + th, bx:bx + tw]
                    t[:sub.shape[0], :sub.shape[1]] = sub
                    blocks.append(t)
        else:
            r = rps or h
            blocks = [a[y:y + r] for y in range(0, h, r)]
        enc = []
        for b in blocks:
            if predictor == 2:
                b = b.copy()
                b[:, 1:] = (b[:, 1:].astype(np.int64) - b[:, :-1].astype(np.int64)).astype(b.dtype)
            raw = b.tobytes()
            enc.append(raw if comp == 1 else packbits(raw) if comp == 32773 else lzw(raw) if comp == 5
                       else zlib.compress(raw))
        if raw_blocks is not None:
            enc = raw_blocks
        offs = []
        for e in enc:
            offs.append(len(out))
            out += e
            if len(out) % 2:
                out += b"\x00"
        entries = [(256, 4, [w]), (257, 4, [h]), (258, 3, [bps]), (259, 3, [comp]), (262, 3, [1]),
                   (277, 3, [1]), (284, 3, [1]), (339, 3, [fmt])]
        if predictor != 1:
            entries.append((317, 3, [predictor]))
        if tile:
            entries += [(322, 4, [tile[0]]), (323, 4, [tile[1]]), (324, 4, offs), (325, 4, [len(e) for e in enc])]
        else:
            entries += [(273, 4, offs), (278, 4, [rps or h]), (279, 4, [len(e) for e in enc])]
        entries.sort()
        ext = {}
        for tag, typ, vals in entries:
            if len(vals) * (2 if typ == 3 else 4) > 4:
                ext[tag] = len(out)
                out += struct.pack(order + ("H" if typ == 3 else "I") * len(vals), *vals)
                if len(out) % 2:
                    out += b"\x00"
        ifd = len(out)
        struct.pack_into(order + "I", out, link, ifd)
        out += struct.pack(order + "H", len(entries))
        for tag, typ, vals in entries:
            out += struct.pack(order + "HHI", tag, typ, len(vals))
            if tag in ext:
                out += struct.pack(order + "I", ext[tag])
            elif typ == 3:
                out += struct.pack(order + "HH", vals[0], 0)
            else:
                out += struct.pack(order + "I", vals[0])
        link = len(out)
        out += b"\x00\x00\x00\x00"
    with open(path, "wb") as f:
        f.write(out)


def test_packbits_example_of_the_specification(wapmod, tmp_path):
    packed = bytes.fromhex("FEAA02800 02AFDAA0380002A22F7AA".replace(" ", ""))
    want = bytes.fromhex("AAAAAA80002AAAAAAAAA80002A22" + "AA" * 10)
    p = str(tmp_path / "pb.tif")
    write_tiff(p, [np.zeros((1, len(want)), np.uint8)], comp=32773, raw_blocks=[packed])
    got = wapmod.tiff_load(p)
    assert np.array_equal(got[0, 0], np.frombuffer(want, np.uint8).astype(np.float32))


def test_lzw_example_of_the_specification(wapmod, tmp_path):
    # the input 7 7 7 8 8 7 7 6 6 codes as Clear 7 258 8 8 258 6 6 End in 9 bits
    codes = pack_codes([(c, 9) for c in (256, 7, 258, 8, 8, 258, 6, 6, 257)])
    assert lzw(bytes([7, 7, 7, 8, 8, 7, 7, 6, 6])) == codes
    p = str(tmp_path / "lzw.tif")
    write_tiff(p, [np.zeros((1, 9), np.uint8)], comp=5, raw_blocks=[codes])
    assert np.array_equal(wapmod.tiff_load(p)[0, 0], np.array([7, 7, 7, 8, 8, 7, 7, 6, 6], np.float32))


@pytest.mark.parametrize("dtype", list(TYPES))
@pytest.mark.parametrize("order", ["<", ">"])
def test_sample_types_and_byte_orders(wapmod, tmp_path, dtype, order):
    rng = np.random.default_rng(1)
    if np.issubdtype(dtype, np.floating):
        pages = [rng.normal(size=(13, 17)).astype(dtype) * 1e3 for _ in range(3)]
    else:
        info = np.iinfo(dtype)
        pages = [rng.integers(info.min, info.max, size=(13, 17), dtype=dtype, endpoint=True) for _ in range(3)]
    p = str(tmp_path / "s.tif")
    write_tiff(p, pages, order=order, rps=5)
    dims, bits, fmt = wapmod.tiff_info(p)
    assert dims == (17, 13, 3, 1) and (bits, fmt) == TYPES[dtype]
    got = wapmod.tiff_load(p)
    assert np.array_equal(got, np.stack(pages).astype(np.float32))


@pytest.mark.parametrize("comp", [1, 32773, 5, 8])
@pytest.mark.parametrize("layout", ["strips", "tiles"])
@pytest.mark.parametrize("predictor", [1, 2])
def test_compressions_layouts_and_predictor(wapmod, tmp_path, comp, layout, predictor):
    rng = np.random.default_rng(comp + predictor)
    # smooth-ish 16-bit data of the size that drives LZW through every code width and a table reset
    y, x = np.mgrid[0:70, 0:150]
    pages = [((np.sin(x / 7.0 + k) * 2000 + y * 40 + rng.integers(0, 300, size=x.shape)) % 65536).astype(np.uint16)
             for k in range(4)]
    p = str(tmp_path / "c.tif")
    write_tiff(p, pages, order=">" if comp == 5 else "<", comp=comp, rps=16 if layout == "strips" else None,
               tile=(64, 32) if layout == "tiles" else None, predictor=predictor)
    got = wapmod.tiff_load(p)
    assert np.array_equal(got, np.stack(pages).astype(np.float32))


def test_lzw_long_run_through_all_code_widths(wapmod, tmp_path):
    rng = np.random.default_rng(7)
    img = rng.integers(0, 4, size=(256, 256), dtype=np.uint8)  # 64 KB: many table resets
    assert len(lzw(img.tobytes())) > 0
    p = str(tmp_path / "big.tif")
    write_tiff(p, [img], comp=5)
    assert np.array_equal(wapmod.tiff_load(p)[0], img.astype(np.float32))


def test_malformed_files_are_refused(wapmod, tmp_path):
    p = str(tmp_path / "ok.tif")
    write_tiff(p, [np.arange(64, dtype=np.uint16).reshape(8, 8)])
    data = open(p, "rb").read()
    bad = [b"", b"II*\x00", b"XX*\x00" + data[4:], data[:2] + b"+\x00" + data[4:], data[:len(data) // 2]]
    for k, b in enumerate(bad):
        q = str(tmp_path / ("bad%d.tif" % k))
        with open(q, "wb") as f:
            f.write(b)
        with pytest.raises(wapmod.WapError):
            wapmod.tiff_load(q)
    with pytest.raises(wapmod.WapError):
        wapmod.tiff_load(str(tmp_path / "missing.tif"))


def test_oversized_header_is_refused_before_allocation(wapmod, tmp_path):
    """A header that claims a page of 2^30 x 8 pixels (far more than the file
    holds) is WAP_ETOOBIG (6) from wap_tiff_info, before any page buffer is
    allocated."""
    import struct
    p = str(tmp_path / "ok.tif")
    write_tiff(p, [np.arange(64, dtype=np.uint16).reshape(8, 8)])
    data = bytearray(open(p, "rb").read())
    ifd = struct.unpack_from("<I", data, 4)[0]
    n = struct.unpack_from("<H", data, ifd)[0]
    for i in range(n):
        e = ifd + 2 + 12 * i
        tag, typ = struct.unpack_from("<HH", data, e)
        if tag == 256:  # ImageWidth, rewritten as a LONG of 2^30
            struct.pack_into("<HHII", data, e, 256, 4, 1, 1 << 30)
    q = str(tmp_path / "huge.tif")
    with open(q, "wb") as f:
        f.write(bytes(data))
    with pytest.raises(wapmod.WapError, match="status 6"):
        wapmod.tiff_info(q)
