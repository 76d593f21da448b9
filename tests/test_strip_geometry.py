"""Launch geometry of the fused multigrid kernels, checked on the host
without a GPU through cf_test_strip_geometry: for every level shape, frame
tiles and register strips together cover the level, every strip reads only
cells in [1, n-1) on both axes (its loads need no bounds checks), the row
count of a strip fits the unrolled row loop, the frame-block numbering is a
bijection onto the tiles outside the strip-covered rectangle, and the block
count is what the kernels index."""
import ctypes
import itertools

import numpy as np
import pytest

from cajitafluids_gb300 import _lib as L

SIZES = [136, 140, 200, 255, 256, 260, 300, 511, 512, 1000, 1024, 1030, 1088, 2048, 2100, 2176, 4096]
SHAPES = sorted(set(itertools.product(SIZES[::2], SIZES[1::2])) | {(n, n) for n in SIZES}
                | {(4096, 2048), (2176, 1088), (2100, 1100), (8192, 8192), (8192, 4096)})


def geometry(nx, ny, tw, th, strip_rows, pre):
    lib = L.load()
    f = (ctypes.c_int * L.CF_STRIP_FIELDS)()
    rc = lib.cf_test_strip_geometry(nx, ny, tw, th, strip_rows, int(pre), f, None, 0)
    assert rc == L.CF_OK
    g = dict(zip(["nframe", "ntx", "txa", "txb", "tya", "tyb", "ns", "nr", "rh", "x0", "y0", "out", "hc", "hr",
                  "cols", "unroll", "per_block", "blocks"], list(f)))
    xy = (ctypes.c_int * (2 * max(g["nframe"], 1)))()
    rc = lib.cf_test_strip_geometry(nx, ny, tw, th, strip_rows, int(pre), f, xy, g["nframe"])
    assert rc == L.CF_OK
    g["frame"] = np.array(list(xy), dtype=np.int64)[:2 * g["nframe"]].reshape(-1, 2)
    return g


def check(nx, ny, tw, th, strip_rows, pre):
    g = geometry(nx, ny, tw, th, strip_rows, pre)
    ntx, nty = -(-nx // tw), -(-ny // th)
    assert g["ntx"] == ntx
    strips = g["ns"] * g["nr"]
    inner = np.zeros((nty, ntx), dtype=bool)
    if strips:
        ns, nr, rh, x0, y0 = g["ns"], g["nr"], g["rh"], g["x0"], g["y0"]
        out, hc, hr = g["out"], g["hc"], g["hr"]
        assert g["cols"] == out + 2 * hc
        # reads of every strip stay in [1, n - 1) on both axes
        assert x0 - hc >= 1 and x0 - hc + out * (ns - 1) + g["cols"] <= nx - 1
        assert y0 - hr >= 1 and y0 + rh * nr + hr <= ny - 1
        # the row loop walks rh + 2 hr rows in whole unrolled trips
        assert rh >= 2 and (rh + 2 * hr) % g["unroll"] == 0
        assert abs(rh - strip_rows) <= g["unroll"] // 2 or rh - g["unroll"] < 2
        # tiles left to the strips lie wholly inside the strip-written cells
        xb, yb = x0 + out * ns, y0 + rh * nr
        assert g["txa"] < g["txb"] and g["tya"] < g["tyb"]
        assert g["txa"] * tw >= x0 and g["txb"] * tw <= xb
        assert g["tya"] * th >= y0 and g["tyb"] * th <= yb
        inner[g["tya"]:g["tyb"], g["txa"]:g["txb"]] = True
    else:
        assert g["nframe"] == ntx * nty
    # frame blocks: a bijection onto the tiles outside the strip rectangle
    fr = g["frame"]
    assert len(fr) == g["nframe"] == ntx * nty - int(inner.sum())
    assert (fr[:, 0] >= 0).all() and (fr[:, 0] < ntx).all() and (fr[:, 1] >= 0).all() and (fr[:, 1] < nty).all()
    hit = np.zeros((nty, ntx), dtype=np.int64)
    np.add.at(hit, (fr[:, 1], fr[:, 0]), 1)
    assert (hit[~inner] == 1).all() and (hit[inner] == 0).all()
    # blocks launched: frame tiles, then per_block strips per block
    assert g["blocks"] == g["nframe"] + -(-strips // g["per_block"])
    return g


@pytest.mark.parametrize("pre", [True, False])
@pytest.mark.parametrize("strip_rows", [32, 8, 20])
def test_register_strips_cover_the_level(built, pre, strip_rows):
    with_strips = 0
    for nx, ny in SHAPES:
        g = check(nx, ny, 64, 32, strip_rows, pre)
        with_strips += g["ns"] * g["nr"] > 0
    assert with_strips > len(SHAPES) // 2


@pytest.mark.parametrize("pre", [True, False])
def test_tiles_only(built, pre):
    for nx, ny in SHAPES + [(16, 16), (33, 17), (65, 65)]:
        g = check(nx, ny, 32, 16, 0, pre)
        assert g["ns"] * g["nr"] == 0


def test_headline_level_geometry(built):
    """The finest level of the 4096^2 workload: 35 strips of 116 written
    columns (pre) or 34 of 120 (post) per band, strip heights 32 and 34,
    and the CTA counts ncu lists for the two launches."""
    pre = check(4096, 4096, 64, 32, 32, True)
    post = check(4096, 4096, 64, 32, 32, False)
    assert (pre["out"], pre["rh"], pre["hc"], pre["hr"]) == (116, 32, 6, 5)
    assert (post["out"], post["rh"], post["hc"], post["hr"]) == (120, 34, 4, 4)
    assert (pre["ns"], post["ns"]) == (35, 34)
    assert pre["blocks"] == 936 and post["blocks"] == 890


def test_rejects_bad_arguments(built):
    lib = L.load()
    f = (ctypes.c_int * L.CF_STRIP_FIELDS)()
    assert lib.cf_test_strip_geometry(0, 64, 64, 32, 32, 1, f, None, 0) == L.CF_ERR_INVALID
    assert lib.cf_test_strip_geometry(64, 64, 48, 32, 0, 1, f, None, 0) == L.CF_ERR_INVALID
    assert lib.cf_test_strip_geometry(64, 64, 32, 16, 32, 1, f, None, 0) == L.CF_ERR_INVALID
    assert lib.cf_test_strip_geometry(64, 64, 64, 32, 32, 1, None, None, 0) == L.CF_ERR_INVALID
    assert lib.cf_test_strip_geometry(64, 64, 64, 32, 32, 1, f, None, 4) == L.CF_ERR_INVALID
