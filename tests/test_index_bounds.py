"""Index arithmetic of every kernel, checked on the CPU against the buffers.

The kernels address padded arrays (NG = 4 ghost layers), the NGV = 2 ring and
interior arrays.  Each offset formula below restates the one in
csrc/cbns_device.cuh / cbns_kernels.cu / cbns_noalloc.cu; offsets are monotone in
i, j, k, so the extreme offsets a launch can touch are reached at the corners of
its index box plus the stencil reach.  Every one must lie inside its buffer for
every block shape the library accepts (each extent >= NG), including the
smallest and odd ones.
"""
import itertools

import pytest

NG, NGV, NEQ = 4, 2, 5
SHAPES = [(4, 4, 4), (4, 5, 6), (5, 4, 7), (7, 9, 4), (12, 16, 20), (33, 17, 9), (64, 64, 64), (256, 256, 256),
          (1000, 8, 8)]


def geom(IM, JM, KM):
    nx, ny, nz = IM + 2 * NG, JM + 2 * NG, KM + 2 * NG
    rx, ry, rz = IM + 2 * NGV, JM + 2 * NGV, KM + 2 * NGV
    return dict(V=nx * ny * nz, RV=rx * ry * rz, IV=IM * JM * KM, nx=nx, ny=ny, rx=rx, ry=ry)


def pad_off(g, i, j, k):
    return (i + NG) + g["nx"] * ((j + NG) + g["ny"] * (k + NG))


def ring_off(g, i, j, k):
    return (i + NGV) + g["rx"] * ((j + NGV) + g["ry"] * (k + NGV))


def int_off(IM, JM, i, j, k):
    return i + IM * (j + JM * k)


def corners(lo, hi):
    """Corners of the box lo <= (i, j, k) < hi."""
    return itertools.product(*[(lo[d], hi[d] - 1) for d in range(3)])


def span(f, lo, hi, reach):
    vals = [f(*c) + r for c in corners(lo, hi) for r in reach]
    return min(vals), max(vals)


@pytest.mark.parametrize("shape", SHAPES)
def test_stage_kernels_stay_in_bounds(shape):
    IM, JM, KM = shape
    g = geom(IM, JM, KM)
    strides = [1, g["nx"], g["nx"] * g["ny"]]
    interior = ((0, 0, 0), (IM, JM, KM))
    # k_inviscid<D>: Q/U at c + m*st, m in -3..2 (SoA, per component n*V + off); prims at c, c - st.
    for st in strides:
        lo, hi = span(lambda i, j, k: pad_off(g, i, j, k), *interior, [m * st for m in range(-3, 3)])
        assert lo >= 0 and hi < g["V"]
    # k_inviscid_x2<1> (binary32 y faces, rows j and j+1 of a thread): the partner row
    # j+1 is always read, the ghost row JM when JM is odd (not stored): its stencil
    # c + m*st, m in -3..2, and its two side cells
    partner = ((0, 1, 0), (IM, JM + 1, KM))
    lo, hi = span(lambda i, j, k: pad_off(g, i, j, k), *partner, [m * strides[1] for m in range(-3, 3)])
    assert lo >= 0 and hi < g["V"]
    # face fluxes: interior offsets and the periodic neighbour (wrapped)
    lo, hi = span(lambda i, j, k: int_off(IM, JM, i, j, k), *interior, [0])
    assert lo >= 0 and hi < g["IV"]
    # FP32-mixed face fluxes (Ff[d], 5 IV floats): equations 0-3 as float4 element
    # f (floats 4 f .. 4 f + 3), equation 4 at float 4 IV + f
    IV = g["IV"]
    assert 4 * lo >= 0 and 4 * hi + 3 < 4 * IV
    assert 4 * IV + lo >= 4 * IV and 4 * IV + hi < 5 * IV
    # k_viscous: ring points i in [-NGV, IM+NGV); derivatives reach +-2 in each direction
    ring = ((-NGV, -NGV, -NGV), (IM + NGV, JM + NGV, KM + NGV))
    for st in strides:
        lo, hi = span(lambda i, j, k: pad_off(g, i, j, k), *ring, [-2 * st, 2 * st])
        assert lo >= 0 and hi < g["V"]
    lo, hi = span(lambda i, j, k: ring_off(g, i, j, k), *ring, [0])
    assert lo >= 0 and hi < g["RV"]
    # k_update: viscous flux stencil at interior cells, +-2 ring strides.  Binary64:
    # term t at t*RV + r (9 blocks); FP32-mixed: the terms differenced along d
    # grouped in block d of 3, one float4 at d*RV + r.
    for d, st in enumerate([1, g["rx"], g["rx"] * g["ry"]]):
        lo, hi = span(lambda i, j, k: ring_off(g, i, j, k), *interior, [-2 * st, 2 * st])
        assert lo >= 0 and hi < g["RV"]
        assert d * g["RV"] + lo >= d * g["RV"] and d * g["RV"] + hi < 3 * g["RV"]
        assert 8 * g["RV"] + hi < 9 * g["RV"]
    # k_update ghost images: i + IM when i < NG, i - IM when i >= IM - NG (per axis)
    for i in range(IM):
        for img in [i] + ([i + IM] if i < NG else []) + ([i - IM] if i >= IM - NG else []):
            assert -NG <= img < IM + NG
    # every ghost cell is the image of exactly one interior cell (x axis; y, z alike)
    for gi in list(range(-NG, 0)) + list(range(IM, IM + NG)):
        sources = [i for i in range(IM) if (i < NG and i + IM == gi) or (i >= IM - NG and i - IM == gi)]
        assert len(sources) == 1
    # k_prepare: the padded box, sources wrapped into the interior
    lo, hi = span(lambda i, j, k: pad_off(g, i, j, k), (-NG, -NG, -NG), (IM + NG, JM + NG, KM + NG), [0])
    assert lo == 0 and hi == g["V"] - 1
    # SoA component bases
    assert (NEQ - 1) * g["V"] + g["V"] - 1 < NEQ * g["V"]


@pytest.mark.parametrize("shape", SHAPES)
def test_diagnostics_and_noalloc_stay_in_bounds(shape):
    IM, JM, KM = shape
    g = geom(IM, JM, KM)
    strides = [1, g["nx"], g["nx"] * g["ny"]]
    for st in strides:
        lo, hi = span(lambda i, j, k: pad_off(g, i, j, k), (0, 0, 0), (IM, JM, KM), [-2 * st, 2 * st])
        assert lo >= 0 and hi < g["V"]
        # the allocation-free entry point reads the reference's AoS layout: 5*c + n
        assert NEQ * lo >= 0 and NEQ * hi + NEQ - 1 < NEQ * g["V"]


def test_tiles_cover_each_domain_exactly():
    """Tiles of 32 x rows cells: guards drop the overhang, nothing is missed."""
    for (ex, ey, ez), rows in itertools.product([(4, 5, 6), (33, 17, 9), (260, 260, 3)], (2, 4, 8)):
        tx, ty = -(-ex // 32), -(-ey // rows)
        covered = set()
        for tk, tj, ti in itertools.product(range(ez), range(ty), range(tx)):
            for t in range(32 * rows):
                i, j = ti * 32 + t % 32, tj * rows + t // 32
                if i < ex and j < ey:
                    covered.add((i, j, tk))
        assert len(covered) == ex * ey * ez
        assert tx < 2 ** 16 and ty < 2 ** 16 and ez < 2 ** 16  # TileRef fields are 16-bit


def test_paired_face_kernel_covers_each_face_once():
    """k_inviscid_x2: threads of 32 x rows/2 over the same tiles, each taking
    rows j and j+1; the partner lane of an odd last row repeats row j and is not
    stored.  Every interior face is stored exactly once, and every cell a lane
    reads (its row's, or the repeated one's) lies in the interior."""
    for (ex, ey, ez), rows in itertools.product([(4, 5, 6), (33, 17, 9), (64, 7, 3), (260, 260, 2)], (2, 4, 8)):
        tx, ty = -(-ex // 32), -(-ey // rows)
        stored = {}
        for tk, tj, ti in itertools.product(range(ez), range(ty), range(tx)):
            for t in range(32 * rows // 2):
                i, j = ti * 32 + t % 32, tj * rows + 2 * (t // 32)
                if i >= ex or j >= ey:
                    continue
                pair = j + 1 < ey
                lanes = [(i, j, tk), (i, j + 1 if pair else j, tk)]
                for c in lanes:
                    assert 0 <= c[0] < ex and 0 <= c[1] < ey and 0 <= c[2] < ez
                for c in lanes[:1 + pair]:
                    stored[c] = stored.get(c, 0) + 1
        assert len(stored) == ex * ey * ez and set(stored.values()) == {1}


def test_plane_tiles_cover_each_ring_exactly():
    """Binary64 k_viscous walks the NGV ring (rx x ry x rz points, rx = IM + 2*NGV) in
    plane tiles: tile q of plane k covers the flattened points p = q*32*rows + t
    of that plane, with j = p // rx, i = p % rx; points past rx*ry are dropped.
    Every ring point is visited exactly once and q fits the split 16-bit fields."""
    for (IM, JM, KM), rows in itertools.product([(4, 5, 6), (33, 17, 9), (64, 7, 3), (256, 256, 2)], (2, 4, 8)):
        rx, ry, rz = IM + 2 * NGV, JM + 2 * NGV, KM + 2 * NGV
        per = 32 * rows
        nq = -(-(rx * ry) // per)
        assert nq < 2 ** 32 and rz < 2 ** 16
        seen = {}
        for k in range(rz):
            for q in range(nq):
                ti, tj = q & 0xFFFF, q >> 16
                first = (ti + 65536 * tj) * per
                for t in range(per):
                    p = first + t
                    if p >= rx * ry:
                        continue
                    j, i = divmod(p, rx)
                    c = (i - NGV, j - NGV, k - NGV)
                    assert -NGV <= c[0] < IM + NGV and -NGV <= c[1] < JM + NGV
                    seen[c] = seen.get(c, 0) + 1
        assert len(seen) == rx * ry * rz and set(seen.values()) == {1}


@pytest.mark.parametrize("shape", SHAPES)
def test_float_float_packed_layouts_stay_in_bounds(shape):
    """CBNS_FP64_FF packs a face's five flux pairs as three float4 per interior
    cell (FFa[d]: element 3 c + h, 3 IV elements) and, per direction, the four
    viscous terms differenced along it as two float4 per ring point (TvG: element
    2 (d RV + r) + h, 6 RV elements).  The update reads the cell's and its
    periodic neighbour's face words and the terms at r +- 1, 2 ring strides; the
    face and viscous kernels write the cell's words and every ring point's."""
    IM, JM, KM = shape
    g = geom(IM, JM, KM)
    IV, RV = g["IV"], g["RV"]
    interior = ((0, 0, 0), (IM, JM, KM))
    ring = ((-NGV, -NGV, -NGV), (IM + NGV, JM + NGV, KM + NGV))
    # FFa: the cell (and, wrapped, its neighbour, also an interior cell) times 3, + 0..2
    lo, hi = span(lambda i, j, k: 3 * int_off(IM, JM, i, j, k), *interior, [0, 1, 2])
    assert lo >= 0 and hi < 3 * IV
    # TvG reads: per direction d, 2 (d RV + r + o) + h, o in +-1, +-2 ring strides
    rstrides = [1, g["rx"], g["rx"] * g["ry"]]
    for d, st in enumerate(rstrides):
        offs = [2 * (d * RV + m * st) + h for m in (-2, -1, 1, 2) for h in (0, 1)]
        lo, hi = span(lambda i, j, k: 2 * ring_off(g, i, j, k), *interior, offs)
        assert lo >= 0 and hi < 6 * RV
    # TvG writes: every ring point, every direction
    lo, hi = span(lambda i, j, k: 2 * ring_off(g, i, j, k), *ring, [2 * d * RV + h for d in range(3) for h in (0, 1)])
    assert lo >= 0 and hi < 6 * RV
    # each direction's block stays in its own third: d RV <= d RV + r +- 2 st < (d + 1) RV
    for st in rstrides:
        lo, hi = span(lambda i, j, k: ring_off(g, i, j, k), *interior, [-2 * st, 2 * st])
        assert lo >= 0 and hi < RV
