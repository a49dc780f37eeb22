"""CPU checks of the kernels' exact arithmetic (host build of the same source), no GPU needed.

chain_add replaces the reference's per-quad accumulation of depth and weights
(Source/DFPSR/implementation/render/shader/fillerTemplates.h:196-244) by a closed
form; it must equal the serial binary32 loop bit for bit.  The row intervals must
equal the oracle's literal restatement of cutConvexEdge (ITriangle2D.cpp:86-169).
"""
import ctypes as C

import numpy as np
import pytest


@pytest.fixture(scope="module")
def host(built):
    from dfpsr_gb300 import build as b
    return C.CDLL(b.HOSTCHECK_LIB)


def _chain(host, s, d, n):
    out = np.zeros_like(s)
    host.dsrg_host_chain_add(C.c_void_p(s.ctypes.data), C.c_void_p(d.ctypes.data), C.c_void_p(n.ctypes.data),
                             C.c_void_p(out.ctypes.data), C.c_int64(len(s)))
    return out


def _serial(s, d, n):
    out = s.copy()
    for i in range(int(n.max()) if len(n) else 0):
        act = i < n
        out[act] = (out[act] + d[act]).astype(np.float32)
    return out


CASES = {
    "depth_like": lambda r, N: (r.uniform(0.2, 0.6, N), r.uniform(-1e-3, 1e-3, N), r.integers(0, 600, N)),
    "weights_cross_zero": lambda r, N: (r.uniform(-1, 1, N), r.uniform(-5e-3, 5e-3, N), r.integers(0, 600, N)),
    "ties": lambda r, N: (r.uniform(1, 2, N), np.ldexp(r.integers(-64, 64, N) * 2 + 1, r.integers(-30, -18, N)), r.integers(0, 400, N)),
    "wide_range": lambda r, N: (r.standard_normal(N) * np.exp(r.uniform(-20, 5, N)), r.standard_normal(N) * np.exp(r.uniform(-25, 2, N)), r.integers(0, 300, N)),
    "binade_edges": lambda r, N: (np.ldexp(1.0, r.integers(-10, 10, N)) * r.choice([1, -1], N) * (1 + r.integers(-3, 3, N) * 2.0 ** -23),
                                  np.ldexp(1.0, r.integers(-40, -1, N)) * r.choice([1, -1], N) * r.uniform(0.5, 1.5, N), r.integers(0, 300, N)),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_chain_add_matches_serial_binary32(host, case):
    r = np.random.default_rng(sum(map(ord, case)))
    s, d, n = CASES[case](r, 40000)
    s, d, n = s.astype(np.float32), d.astype(np.float32), n.astype(np.int32)
    a, b = _chain(host, s, d, n), _serial(s, d, n)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_chain_add_special_values(host):
    s = np.array([0.0, -0.0, 1e-40, np.inf, np.nan, 1.0, 3.4e38, -1.0], np.float32)
    d = np.array([1e-3, -1e-3, 1e-41, 1.0, 1.0, np.inf, 3e37, 1e-30], np.float32)
    n = np.array([5, 5, 50, 3, 3, 2, 4, 1000], np.int32)
    a, b = _chain(host, s, d, n), _serial(s, d, n)
    same = (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))
    assert same.all()


def _rows(host, flat, y0, rows, L, R):
    fl = np.ascontiguousarray(flat, np.int32)
    lefts, rights = np.zeros(rows, np.int32), np.zeros(rows, np.int32)
    host.dsrg_host_row_intervals(C.c_void_p(fl.ctypes.data), C.c_int32(y0), C.c_int32(rows), C.c_int32(L), C.c_int32(R),
                                 C.c_void_p(lefts.ctypes.data), C.c_void_p(rights.ctypes.data))
    return lefts, rights


def _bound_x(flat, width):
    rx = [int((v + 128) / 256) for v in flat[0::2]]  # C truncating division
    return max(min(rx) - 1, 0), min(max(rx) + 1, width)


@pytest.mark.parametrize("kind", ["random", "near_horizontal", "small", "vertical", "offscreen"])
def test_row_intervals_match_oracle(host, kind):
    from oracle import port
    r = np.random.default_rng(sum(map(ord, kind)))
    W, H = 800, 600
    checked = 0
    for _ in range(1500):
        if kind == "random":
            f = r.integers(-W * 128, W * 384, 6)
        elif kind == "near_horizontal":
            f = r.integers(-300 * 256, 1100 * 256, 6)
            f[1] = f[3] + r.integers(-3, 3)
        elif kind == "small":
            f = r.integers(0, 6 * 256, 6) + r.integers(0, W * 256)
        elif kind == "vertical":
            f = r.integers(-W * 128, W * 384, 6)
            f[0] = f[2]
        else:
            f = np.array([r.integers(-W * 256, -10), r.integers(0, H * 256), r.integers(-W * 256, -10),
                          r.integers(0, H * 256), r.integers(0, W * 256), r.integers(0, H * 256)])
        f = f.astype(np.int64)
        start, L, R = port.triangle_rows(f, [0, 0, W, H])
        if len(L) == 0:
            continue
        lo, hi = _bound_x(f, W)
        lefts, rights = _rows(host, f, start, len(L), lo, hi)
        assert np.array_equal(lefts, L) and np.array_equal(rights, R), f
        checked += 1
    assert checked > 50


@pytest.mark.parametrize("kind", ["random", "near_horizontal", "small", "vertical", "offscreen", "far", "degenerate"])
def test_stepped_row_intervals_equal_per_row_intervals(host, kind):
    """row_intervals_stepped (two int64 divisions per edge, then integer steps) equals row_interval
    of every row, including the empty rows' exact left/right values that row pairs read."""
    r = np.random.default_rng(100 + sum(map(ord, kind)))
    for _ in range(3000):
        if kind == "random":
            f = r.integers(-800 * 128, 800 * 384, 6)
        elif kind == "near_horizontal":
            f = r.integers(-300 * 256, 1100 * 256, 6)
            f[1] = f[3] + r.integers(-3, 3)
        elif kind == "small":
            f = r.integers(0, 6 * 256, 6) + r.integers(0, 800 * 256)
        elif kind == "vertical":
            f = r.integers(-800 * 128, 800 * 384, 6)
            f[0] = f[2]
        elif kind == "offscreen":
            f = np.array([r.integers(-800 * 256, -10), r.integers(0, 600 * 256), r.integers(-800 * 256, -10),
                          r.integers(0, 600 * 256), r.integers(0, 800 * 256), r.integers(0, 600 * 256)])
        elif kind == "far":  # corners up to the records' coordinate limit of 2^30
            f = r.integers(-(1 << 30), 1 << 30, 6)
        else:
            f = r.integers(0, 4 * 256, 6)
            f[2:4] = f[0:2]
        f = np.ascontiguousarray(f.astype(np.int32))
        y0 = int(r.integers(-40, 640))
        rows = int(r.integers(1, 40))
        L, R = int(r.integers(0, 400)), int(r.integers(400, 801))
        a = _rows(host, f, y0, rows, L, R)
        lefts, rights = np.zeros(rows, np.int32), np.zeros(rows, np.int32)
        host.dsrg_host_row_intervals_stepped(C.c_void_p(f.ctypes.data), C.c_int32(y0), C.c_int32(rows), C.c_int32(L), C.c_int32(R),
                                             C.c_void_p(lefts.ctypes.data), C.c_void_p(rights.ctypes.data))
        assert np.array_equal(lefts, a[0]) and np.array_equal(rights, a[1]), (f.tolist(), y0, rows, L, R)
