"""The temporally blocked tiling, emulated on the CPU with the oracle's own updates (no GPU).

The CUDA tiles advance an extended region K steps and keep only its inner part; column segments
step a head tile and then carried tiles that have no top halo and take the Hz row above them
from their predecessor at every step. Both rest on one argument: a cut edge of a region goes
stale, and the error it causes moves at most one cell per step (the H update reads E at +1,
the E update reads Hz at -1). This test restates both schemes with ``oracle.te_numpy``'s
``update_h`` / ``update_e`` on sub-arrays (each one a small simulation whose cut edges stay
unupdated, as outer walls do) and checks that the assembled fields and psi equal the oracle's
whole-grid run bit for bit, with CPML profiles on every edge, point sources and random states.
With the halo one row short, the same assembly differs from the oracle.
"""

from types import SimpleNamespace

import numpy as np
import pytest

from oracle.te_numpy import update_e, update_h

PROFILES = ("bx_e", "cx_e", "ikx_e", "bx_h", "cx_h", "ikx_h", "by_e", "cy_e", "iky_e", "by_h", "cy_h", "iky_h")
# array -> (extra row, extra column) over the Hz shape (nx, ny)
ARRAYS = {"hz": (0, 0), "psi_hz_x": (0, 0), "psi_hz_y": (0, 0), "ex": (0, 1), "psi_ex_y": (0, 1),
          "cb_ex": (0, 1), "ey": (1, 0), "psi_ey_x": (1, 0), "cb_ey": (1, 0)}  # fmt: skip
STATE = ("hz", "psi_hz_x", "psi_hz_y", "ex", "psi_ex_y", "ey", "psi_ey_x")


def random_state(nx, ny, dtype, seed, layers=6):
    """Random fields and psi everywhere, cb in (0.2, 0.5), CPML-like profiles on all four edges."""
    rng = np.random.default_rng(seed)
    s = SimpleNamespace(nx=nx, ny=ny, db=dtype(0.5), inv_dx=dtype(1.0), inv_dy=dtype(1.0))
    for name, (er, ec) in ARRAYS.items():
        shape = (nx + er, ny + ec)
        if name.startswith("cb"):
            a = rng.uniform(0.2, 0.5, shape)
        elif name.startswith("psi"):
            a = 0.05 * rng.standard_normal(shape)
        else:
            a = rng.standard_normal(shape)
        setattr(s, name, a.astype(dtype))
    for name in PROFILES:
        n = (nx if name[1] == "x" or name[2] == "x" else ny) + (1 if name.endswith("_e") else 0)
        b, c, ik = np.ones(n), np.zeros(n), np.ones(n)
        edge = np.r_[0:layers, n - layers : n]
        b[edge] = rng.uniform(0.3, 0.9, edge.size)
        c[edge] = -rng.uniform(0.01, 0.1, edge.size)
        ik[edge] = rng.uniform(0.5, 1.0, edge.size)
        setattr(s, name, {"b": b, "c": c, "i": ik}[name[0]].astype(dtype))
    return s


def sources(nx, ny, k, dtype, seed):
    """(array, i, j, deltas per step): an Hz node and an Ey node, inside and on tile seams."""
    rng = np.random.default_rng(seed + 1)
    return [("hz", nx // 2, ny // 3, rng.standard_normal(k).astype(dtype)),
            ("ey", nx // 3, ny // 2, rng.standard_normal(k).astype(dtype)),
            ("hz", 12, 8, rng.standard_normal(k).astype(dtype))]  # fmt: skip


def step(s, srcs, n, r0=0, c0=0, carry=None):
    """One step of a (sub-)simulation whose arrays start at global cell (r0, c0): H, the magnetic
    sources it holds, the carried Hz row (row 0, if any), E, the electric sources it holds."""
    update_h(s)
    inject(s, srcs, n, r0, c0, magnetic=True)
    if carry is not None:
        s.hz[0, :] = carry
    update_e(s)
    inject(s, srcs, n, r0, c0, magnetic=False)


def inject(s, srcs, n, r0, c0, magnetic):
    for name, i, j, d in srcs:
        if (name == "hz") != magnetic:
            continue
        a = getattr(s, name)
        if 0 <= i - r0 < a.shape[0] and 0 <= j - c0 < a.shape[1]:
            a[i - r0, j - c0] -= d[n]


def sub(g, r0, r1, c0, c1):
    """The small simulation over cell rows [r0, r1) and columns [c0, c1) (clipped to the grid):
    Hz and psi_hz of the cells, Ex with the column after, Ey with the row after; its edges are
    updated as outer walls, which is where a cut region goes stale."""
    r0, c0 = max(r0, 0), max(c0, 0)
    nxs, nys = min(r1, g.nx) - r0, min(c1, g.ny) - c0
    m = SimpleNamespace(nx=nxs, ny=nys, db=g.db, inv_dx=g.inv_dx, inv_dy=g.inv_dy)
    for name, (er, ec) in ARRAYS.items():
        setattr(m, name, getattr(g, name)[r0 : r0 + nxs + er, c0 : c0 + nys + ec].copy())
    for name in PROFILES:
        lo, n = (r0, nxs) if name[1] == "x" or name[2] == "x" else (c0, nys)
        setattr(m, name, getattr(g, name)[lo : lo + n + (1 if name.endswith("_e") else 0)])
    return m, r0, c0


def write_back(dst, m, r0, c0, rows, cols):
    """Copy the cells [rows) x [cols) that the small simulation owns into the global state."""
    for name in STATE:
        a = getattr(dst, name)
        a0, a1 = max(rows[0], 0), min(rows[1], a.shape[0])
        b0, b1 = max(cols[0], 0), min(cols[1], a.shape[1])
        if a1 > a0 and b1 > b0:
            a[a0:a1, b0:b1] = getattr(m, name)[a0 - r0 : a1 - r0, b0 - c0 : b1 - c0]


def blocked(g, srcs, k, er, ec, segments, halo=None, carry_rows=True, shift=0):
    """K steps of the whole grid as tiles of er x ec extended cells (output er - 2K rows, ec - 2K
    columns). With `segments`, each run of five tile rows of a column is one head tile and three
    carried tiles (er - K output rows, no top halo, the Hz row above taken from the predecessor
    after every H update), the scheme of the column-segment kernel; er must then be 5K. The
    first tile column starts at `shift` (<= 0), as the kernels' tile lists may.
    `halo` and `carry_rows` exist to plant mistakes: a shorter halo, carried tiles left alone."""
    h = k if halo is None else halo
    out_r, out_c = er - 2 * k, ec - 2 * k
    new = SimpleNamespace(**{name: getattr(g, name).copy() for name in STATE})
    for c in range(shift, g.ny + 1, out_c):
        cols = (c, c + out_c)
        rows = list(range(0, g.nx + 1, out_r))
        q = 0
        while q < len(rows):
            if segments and q + 5 <= len(rows):
                assert er == 5 * k
                r, carry = rows[q], None
                for u in range(4):
                    own = out_r if u == 0 else er - k
                    top = r - h if u == 0 else r - 1  # a carried tile keeps one row: the carried Hz
                    m, m0, n0 = sub(g, top, r + own + h, c - h, c + out_c + h)
                    rec, next_row = [], r + own - 1  # the predecessor's row above the next tile
                    for n in range(k):
                        step(m, srcs, n, m0, n0, None if carry is None or not carry_rows else carry[n])
                        rec.append(m.hz[next_row - m0, :].copy())
                    write_back(new, m, m0, n0, (r, r + own), cols)
                    carry, r = rec, r + own
                q += 5
            else:
                r = rows[q]
                m, m0, n0 = sub(g, r - h, r + out_r + h, c - h, c + out_c + h)
                for n in range(k):
                    step(m, srcs, n, m0, n0)
                write_back(new, m, m0, n0, (r, r + out_r), cols)
                q += 1
    return new


def whole_grid(g, srcs, k):
    s = SimpleNamespace(**{name: getattr(g, name).copy() for name in ARRAYS})
    for name in ("nx", "ny", "db", "inv_dx", "inv_dy", *PROFILES):
        setattr(s, name, getattr(g, name))
    for n in range(k):
        step(s, srcs, n)
    return s


def same_bits(a, b) -> bool:
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("k", [2, 4])
@pytest.mark.parametrize("segments", [False, True], ids=["tiles", "segments"])
@pytest.mark.parametrize("shift", [0, -5])
def test_blocked_tiles_equal_the_whole_grid_run(dtype, k, segments, shift):
    nx, ny = 67, 45
    g = random_state(nx, ny, dtype, seed=k)
    srcs = sources(nx, ny, k, dtype, seed=k)
    want = whole_grid(g, srcs, k)
    got = blocked(g, srcs, k, er=5 * k, ec=8 + 2 * k, segments=segments, shift=shift)
    for name in STATE:
        assert same_bits(getattr(got, name), getattr(want, name)), name


@pytest.mark.parametrize("segments", [False, True], ids=["tiles", "segments"])
def test_a_halo_one_row_short_is_caught(segments):
    """The check is not vacuous: with a halo of K - 1 cells the stale edges reach the output."""
    nx, ny, k = 67, 45, 4
    g = random_state(nx, ny, np.float32, seed=9)
    srcs = sources(nx, ny, k, np.float32, seed=9)
    want = whole_grid(g, srcs, k)
    got = blocked(g, srcs, k, er=5 * k, ec=8 + 2 * k, segments=segments, halo=k - 1)
    assert not all(same_bits(getattr(got, name), getattr(want, name)) for name in STATE)


def test_carried_tiles_need_the_carried_row():
    """Without the Hz row from their predecessor, carried tiles (no top halo) go wrong."""
    nx, ny, k = 67, 45, 4
    g = random_state(nx, ny, np.float32, seed=5)
    srcs = sources(nx, ny, k, np.float32, seed=5)
    want = whole_grid(g, srcs, k)
    got = blocked(g, srcs, k, er=5 * k, ec=8 + 2 * k, segments=True, carry_rows=False)
    assert not all(same_bits(getattr(got, name), getattr(want, name)) for name in STATE)
