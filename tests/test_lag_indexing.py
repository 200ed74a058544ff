"""Index arithmetic of the one-kernel Lagrangian phase (lag_fused.cuh), checked
on the CPU for many mesh sizes before any of it runs on a GPU.

The tile stages its input rows with TMA bulk copies, which need 16-byte
aligned addresses and sizes and must stay inside the arrays; every thread then
reads its values back at a shared-memory index derived from the copy.  This
test restates that integer arithmetic (make_seg, seg_cells, seg_xfaces,
seg_yfaces and the thread roles of lag_tile) and checks, for every tile, row
and thread of each mesh:

* each copy starts on an even element (16 bytes for an aligned base), has an
  even length no longer than a ring slot, and lies inside its array;
* each shared-memory read lands inside the copied range, on the element the
  thread wants;
* every output store (velocities, changed values, masks) is inside its array,
  and every interior face and cell is produced by exactly one tile.
"""
import itertools

import pytest

KT, KHALO = 128, 3
KW = KT - 2 * KHALO
KSEG = KT + 4
KWARPS = KT // 32
PAD = 2


def make_seg(row_base, clo, chi):
    if clo >= chi:
        return None
    g0 = row_base + clo
    g0a = g0 & ~1
    g1a = (row_base + chi + 1) & ~1
    return g0a, g1a - g0a, clo - (g0 - g0a)


def tile_geom(nx, ny, rows, bx, by):
    cb = PAD + bx * KW
    r0 = PAD + by * rows
    r1 = min(r0 + rows, ny - PAD)
    return cb, r0, r1, r0 - KHALO, r1 + KHALO - 1


def seg_cells(nx, ny, g, i):
    cb, r0, r1, ia, ib = g
    if i < max(r0 - KHALO, 1) or i > min(r1 + KHALO - 1, ny - 2):
        return None
    return make_seg(i * nx, max(cb - KHALO, 1), min(cb - KHALO + KT, nx - 1))


def seg_xfaces(nx, ny, g, i):
    cb, r0, r1, ia, ib = g
    if i < r0 or i >= r1:
        return None
    return make_seg(i * (nx + 1), max(cb - 2, PAD), min(cb + KW + 2, nx - PAD) + 1)


def seg_yfaces(nx, ny, g, i):
    cb, r0, r1, ia, ib = g
    if i < max(r0 - 2, PAD) or i > min(r1 + 2, ny - PAD):
        return None
    return make_seg(i * nx, max(cb, PAD), min(cb + KW, nx - PAD))


def check_seg(seg, alloc):
    if seg is None:
        return
    g0a, n, c0a = seg
    assert g0a % 2 == 0 and n % 2 == 0, seg
    assert 0 < n <= KSEG, seg
    assert g0a >= 0 and g0a + n <= alloc, (seg, alloc)


def read_ok(seg, col):
    g0a, n, c0a = seg
    idx = col - c0a
    assert 0 <= idx < n, (seg, col)
    return idx


def check_mesh(gnx, gny, rows):
    nx, ny = gnx + 2 * PAD, gny + 2 * PAD
    ncell, nface = nx * ny, (nx + 1) * (ny + 1)
    ntx = (nx - 2 * PAD + 1 + KW - 1) // KW
    nty = (ny - 2 * PAD + rows - 1) // rows
    mask_words = nx * ny * 2  # rho_old holds nx*ny doubles
    if (ny + 1) * ntx * 3 * KWARPS > mask_words:
        return False  # the host runs the four-kernel form instead (fused.cu)
    u_owner, v_owner, e_owner = {}, {}, {}
    for bx, by in itertools.product(range(ntx), range(nty)):
        g = tile_geom(nx, ny, rows, bx, by)
        cb, r0, r1, ia, ib = g
        assert ib - ia + 1 <= rows + 2 * KHALO
        for i in range(ia, ib + 1):
            sc, sx, sy = seg_cells(nx, ny, g, i), seg_xfaces(nx, ny, g, i), seg_yfaces(nx, ny, g, i)
            check_seg(sc, ncell)
            check_seg(sx, nface)
            check_seg(sy, nface)
            for t in range(KT):
                c = cb - KHALO + t
                # own cell (phase 1); the kernel forms the shared index from
                # the row parity: col - clo + ((row*len + clo) & 1)
                if sc is not None and 1 <= c <= nx - 2:
                    clo = max(cb - KHALO, 1)
                    assert read_ok(sc, c) == c - clo + (((i & nx) ^ clo) & 1)
                # pressure-phase face (phase 2) and its cells
                fc = None
                if t >= 1:
                    if PAD <= c <= nx - PAD:
                        fc = c
                    elif c == PAD - 1:
                        fc = PAD
                    elif c == nx - PAD + 1:
                        fc = nx - PAD
                if r0 <= i < r1 and fc is not None:
                    clo = max(cb - 2, PAD)
                    assert read_ok(sx, fc) == fc - clo + (((i & (nx + 1)) ^ clo) & 1)
                    tf = fc - (cb - KHALO)
                    assert 1 <= tf < KT
                    # cells fc-1, fc were loaded by threads tf-1, tf
                    assert sc is not None
                    read_ok(sc, fc - 1)
                    read_ok(sc, fc)
                cell_out = max(cb, PAD) <= c < min(cb + KW, nx - PAD)
                if cell_out and max(r0 - 2, PAD) <= i <= min(r1 + 2, ny - PAD):
                    clo = max(cb, PAD)
                    assert read_ok(sy, c) == c - clo + (((i & nx) ^ clo) & 1)
        # outputs
        for t in range(KT):
            c = cb - KHALO + t
            uf_out = max(cb, PAD) <= c <= min(cb + KW, nx - PAD) and c < cb + KW
            cell_out = max(cb, PAD) <= c < min(cb + KW, nx - PAD)
            q_role = max(cb - 1, PAD) <= c <= min(cb + KW, nx - PAD - 1)
            uf_role = max(cb, PAD) <= c <= min(cb + KW, nx - PAD)
            if q_role:
                assert 2 <= t <= KT - 3
            if uf_role:
                assert 1 <= t <= KT - 2
            for row in range(r0, r1):
                if uf_out:
                    f = row * (nx + 1) + c
                    assert 0 <= f < nface
                    assert (row, c) not in u_owner
                    u_owner[(row, c)] = (bx, by)
                if cell_out:
                    ci = row * nx + c
                    assert 0 <= ci < ncell
                    assert (row, c) not in e_owner
                    e_owner[(row, c)] = (bx, by)
            vrows = list(range(r0, r1)) + ([r1] if r1 == ny - PAD else [])
            for row in vrows:
                if cell_out:
                    assert (row, c) not in v_owner
                    v_owner[(row, c)] = (bx, by)
        for row in range(r0, r1 + 1):
            for field in range(3):
                base = ((row * ntx + bx) * 3 + field) * KWARPS
                assert base + KWARPS <= (ny + 1) * ntx * 3 * KWARPS
    # every interior point produced exactly once
    assert set(u_owner) == {(r, c) for r in range(PAD, ny - PAD) for c in range(PAD, nx - PAD + 1)}
    assert set(e_owner) == {(r, c) for r in range(PAD, ny - PAD) for c in range(PAD, nx - PAD)}
    assert set(v_owner) == {(r, c) for r in range(PAD, ny - PAD + 1) for c in range(PAD, nx - PAD)}
    return True


SIZES = [(2, 2), (3, 5), (7, 3), (24, 20), (40, 40), (96, 80), (121, 37), (122, 64),
         (123, 65), (151, 93), (244, 130), (245, 129), (512, 512)]


@pytest.mark.parametrize("gnx,gny", SIZES)
@pytest.mark.parametrize("rows", [1, 5, 16, 32, 64])
def test_lagrangian_tile_indexing(gnx, gny, rows):
    fused = check_mesh(gnx, gny, rows)
    assert fused or gnx * gny < 64
