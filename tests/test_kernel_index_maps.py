"""Index arithmetic of the HBM-bound kernels, restated in Python (CPU).

kernels_fp64.cu: canonical_axes (unit axes dropped, neighbours contiguous in both tensors
merged), the row-segment permute (128-element segments of the last output axis, a
contiguous range of segments per warp), the 32 x 32 tile permute, and the tiled (T)
energy kernel's closed-form tile indices (thread t, iteration it -> element t + 128 it).
Each mapping must visit exactly the (input offset, output offset) pairs of the direct
enumeration, once each, inside the tensors."""
import itertools
import random

import pytest


def canonical(od, is_, os_):
    d, i, o = [], [], []
    for k in range(len(od)):
        if od[k] == 1:
            continue
        if d and i[-1] == is_[k] * od[k] and o[-1] == os_[k] * od[k]:
            d[-1] *= od[k]
            i[-1], o[-1] = is_[k], os_[k]
            continue
        d.append(od[k]), i.append(is_[k]), o.append(os_[k])
    return (d, i, o) if d else ([1], [1], [1])


def direct(od, is_, os_):
    return sorted((sum(a * b for a, b in zip(ix, is_)), sum(a * b for a, b in zip(ix, os_)))
                  for ix in itertools.product(*[range(x) for x in od]))


def rows_map(d, i, o, nwarps):
    r, dl = len(d), d[-1]
    rows = 1
    for x in d[:-1]:
        rows *= x
    nseg = (dl + 127) // 128
    items = rows * nseg
    per = (items + nwarps - 1) // nwarps
    out = []
    for warp in range(nwarps):
        for w in range(warp * per, min(warp * per + per, items)):
            row, x0 = w // nseg, (w % nseg) * 128
            rem, bi, bo = row, 0, 0
            for k in range(r - 2, -1, -1):
                x = rem % d[k]
                rem //= d[k]
                bi += x * i[k]
                bo += x * o[k]
            out += [(bi + x * i[-1], bo + x * o[-1]) for x in range(x0, min(x0 + 128, dl))]
    return sorted(out)


def tile_map(d, i, o, q):
    r, dl, dq = len(d), d[-1], d[q]
    rest = [k for k in range(r - 1) if k != q]
    out = []
    for rr in itertools.product(*[range(d[k]) for k in rest]):
        bi = sum(x * i[k] for x, k in zip(rr, rest))
        bo = sum(x * o[k] for x, k in zip(rr, rest))
        for tq in range(0, dq, 32):
            for tl in range(0, dl, 32):
                for jj in range(32):
                    for tx in range(32):
                        xq, xl = tq + jj, tl + tx
                        if xl < dl and xq < dq:
                            out.append((bi + xq * i[q] + xl * i[-1], bo + xq * o[q] + xl * o[-1]))
    return sorted(out)


def test_permute_maps_cover_every_element_once():
    random.seed(0)
    for _ in range(150):
        rank = random.randint(1, 4)
        dims = [random.choice([1, 2, 3, 5, 8, 9, 33, 40]) for _ in range(rank)]
        perm = list(range(rank))
        random.shuffle(perm)
        st, acc = [0] * rank, 1
        for k in range(rank - 1, -1, -1):
            st[perm[k]] = acc
            acc *= dims[perm[k]]
        os_, acc, pad = [0] * rank, 1, random.choice([0, 0, 3])
        for k in range(rank - 1, -1, -1):
            os_[k] = acc
            acc *= dims[k] + (pad if k == rank - 1 else 0)
        ref = direct(dims, st, os_)
        d, i, o = canonical(dims, st, os_)
        assert direct(d, i, o) == ref
        r = len(d)
        q = -1
        if r >= 2 and i[-1] != 1 and o[-1] == 1 and d[-1] >= 8:
            for k in range(r - 1):
                if i[k] == 1 and d[k] >= 8:
                    q = k
        if q >= 0:
            assert tile_map(d, i, o, q) == ref
        elif d[-1] >= 32:
            assert rows_map(d, i, o, random.choice([1, 3, 8, 1000])) == ref


def test_full_copy_merges_to_one_axis_and_spreads_over_warps():
    d, i, o = canonical([16, 16, 160, 160], [409600, 25600, 160, 1], [409600, 25600, 160, 1])
    assert (d, i, o) == ([16 * 16 * 160 * 160], [1], [1])
    # 6.5M elements as 128-element segments over a 19456-warp grid: most warps get a share
    items = (d[0] + 127) // 128
    per = (items + 19455) // 19456
    busy = (items + per - 1) // per
    assert busy >= 0.8 * 19456


def test_triples_energy_closed_form_indices():
    ET, NT = 8, 128
    for tid in range(NT):
        tx, ty, tz = tid // (ET * ET), (tid // ET) % ET, tid % ET
        for it in range(6 * ET ** 3 // NT):  # the six permutation tiles of W3
            e = tid + NT * it
            p, rem = divmod(e, ET ** 3)
            assert (p, rem // (ET * ET), (rem // ET) % ET, rem % ET) == (it // 4, tx + 2 * (it % 4), ty, tz)
        for it in range(3 * 6 * ET * ET // NT):  # Vij, Vik, Vjk on the six ordered role pairs
            e = tid + NT * it
            m, rem = divmod(e, 6 * ET * ET)
            pid = rem // (ET * ET)
            assert (m, pid, pid // 2, pid % 2, (rem // ET) % ET, rem % ET) == (it // 3, 2 * (it % 3) + tx, it % 3,
                                                                               tx, ty, tz)
        for it in range(ET ** 3 // NT):  # the energy loop
            q = tid + NT * it
            assert (q // (ET * ET), (q // ET) % ET, q % ET) == (tx + 2 * it, ty, tz)


def _raster(mgroups, ntiles, tl, band_n=8):
    """The tensor-core GEMMs' raster order (tc_gemm.cu raster()): bands of band_n N tiles,
    M groups in order inside a band, the band's N tiles fastest."""
    band = tl // (mgroups * band_n)
    w = min(band_n, ntiles - band * band_n)
    r = tl - band * mgroups * band_n
    mg = r // w
    return mg, band * band_n + (r - mg * w)


@pytest.mark.parametrize("mgroups,ntiles", [(1, 1), (40, 40), (40, 2), (3, 17), (80, 9), (7, 8), (1, 13)])
def test_raster_order_visits_every_tile_once(mgroups, ntiles):
    seen = [_raster(mgroups, ntiles, t) for t in range(mgroups * ntiles)]
    assert sorted(seen) == [(m, n) for m in range(mgroups) for n in range(ntiles)]
    # tiles in flight together (a window of 152) share operands: at most ~8 N tiles span it
    # whenever there are that many M groups
    if mgroups >= 19 and ntiles >= 8:
        window = seen[:152]
        assert len({n for _, n in window}) <= 8 and len({m for m, _ in window}) <= 19


# ---- blocked W3 layout of the mixed (T) path (core.h w3_block_offset) ----------------
def w3_block_offset(a, b, c, T):
    x, y, z = a & 7, b & 7, c & 7
    return (((a >> 3) * T + (b >> 3)) * T + (c >> 3)) * 512 + 64 * x + 8 * (y ^ x) + (z ^ ((5 * y) & 7))


@pytest.mark.parametrize("nv", [8, 20, 84])
def test_w3_block_layout_is_a_bijection_onto_whole_blocks(nv):
    T = (nv + 7) // 8
    offs = [w3_block_offset(a, b, c, T) for a in range(8 * T) for b in range(8 * T) for c in range(8 * T)]
    assert sorted(offs) == list(range(T ** 3 * 512))
    # a tile (A, B, C) of the energy kernel is exactly block (A, B, C): 512 contiguous floats
    for A, B, C in [(0, 0, 0), (T - 1, 0, T - 1), (T - 1, T - 1, T - 1)]:
        blk = {w3_block_offset(8 * A + x, 8 * B + y, 8 * C + z, T)
               for x in range(8) for y in range(8) for z in range(8)}
        base = ((A * T + B) * T + C) * 512
        assert blk == set(range(base, base + 512))


def test_w3_epilogue_fast_path_matches_the_layout():
    """The GEMM epilogue stores 32 columns c = n0 .. n0 + 31 of one (a, b) row as four
    8-wide c blocks, after v[p] <- v[p ^ k] with k = 5 (b % 8) % 8, at base + block * 512."""
    T = 5
    for a, b, n0 in [(0, 0, 0), (13, 29, 0), (39, 7, 32), (22, 31, 0)]:
        x, y, k = a & 7, b & 7, (5 * (b & 7)) & 7
        base = (((a >> 3) * T + (b >> 3)) * T) * 512 + 64 * x + 8 * (y ^ x)
        for g in range(4):
            v = list(range(n0 + 8 * g, n0 + 8 * g + 8))  # the column each register holds
            for bit in (1, 2, 4):  # xor_swap8: three conditional swaps
                if k & bit:
                    for e in range(8):
                        if not e & bit:
                            v[e], v[e | bit] = v[e | bit], v[e]
            for pos, col in enumerate(v):
                assert base + ((n0 >> 3) + g) * 512 + pos == w3_block_offset(a, b, col, T)


def test_energy_thread_order_reads_blocks_without_bank_conflicts():
    """triples_energy_pipe_kernel: 256 threads x 2 iterations cover a tile once, and every
    warp's read of each of the six index orders, and of the Voovv rows, is one wavefront:
    no bank holds two different words (words at 64 x + 8 (y ^ x) + (z ^ 5y), 4-byte banks;
    lanes reading the same word share it)."""
    def wavefronts(words):
        banks = {}
        for x in set(words):
            banks.setdefault(x % 32, set()).add(x)
        return max(len(v) for v in banks.values())

    def elem(tid, it):
        la = (tid & 1) | (((tid >> 6) & 1) << 1) | (((tid >> 7) & 1) << 2)
        lb = ((tid >> 2) & 1) | (((tid >> 1) & 1) << 1) | (((tid >> 5) & 1) << 2)
        lc = ((tid >> 4) & 1) | (((tid >> 3) & 1) << 1) | ((it & 1) << 2)
        return la, lb, lc
    assert len({elem(t, i) for t in range(256) for i in range(2)}) == 512
    orders = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    for it in range(2):
        for w in range(8):
            E = [elem(32 * w + lane, it) for lane in range(32)]
            for o in orders:
                assert wavefronts([w3_block_offset(e[o[0]], e[o[1]], e[o[2]], 1) for e in E]) == 1, (it, w, o)
            for u, v in [(0, 1), (0, 2), (1, 0), (1, 2), (2, 0), (2, 1)]:  # Voovv rows of 8
                assert wavefronts([8 * e[u] + e[v] for e in E]) == 1


def test_w3_epilogue_block_walk_matches_the_layout():
    """Columns that are a or b (or c past the float4 path): block part linear in the
    8-wide block, plus one of eight in-block offsets fixed by the row."""
    T = 5
    for rn in range(3):  # role of the column index: 0 a, 1 b, 2 c
        for rh in range(3):
            if rh == rn:
                continue
            rl = 3 - rn - rh
            for hi, lo, n0 in [(0, 0, 0), (13, 29, 32), (39, 7, 0), (22, 31, 32)]:
                fa = hi if rh == 0 else (lo if rl == 0 else 0)
                fb = hi if rh == 1 else (lo if rl == 1 else 0)
                fc = hi if rh == 2 else (lo if rl == 2 else 0)
                nb0 = n0 >> 3
                bA, bB, bC = (nb0 if rn == 0 else fa >> 3), (nb0 if rn == 1 else fb >> 3), (nb0 if rn == 2 else fc >> 3)
                blk0 = ((bA * T + bB) * T + bC) * 512
                gstride = (T * T if rn == 0 else (T if rn == 1 else 1)) * 512
                for j in range(32):
                    e = j & 7
                    x, y, z = (e if rn == 0 else fa & 7), (e if rn == 1 else fb & 7), (e if rn == 2 else fc & 7)
                    loc = 64 * x + 8 * (y ^ x) + (z ^ ((5 * y) & 7))
                    n = n0 + j
                    abc = [fa, fb, fc]
                    abc[rn] = n
                    assert blk0 + (j >> 3) * gstride + loc == w3_block_offset(*abc, T)


@pytest.mark.parametrize("nx,nv", [(3, 5), (2, 33), (4, 70)])
def test_pack_pairs_tiled_writes_every_packed_element_once(nx, nv):
    """pack_pairs_tiled_kernel: block (tile pair E <= F, row pair x <= y), lanes over e,
    rows over f; every element of P[x<=y][e<=f] and M[x<y][e<f] written once, from the
    right t[e][f] and t[f][e]."""
    import numpy as np
    rng = np.random.default_rng(nx * 100 + nv)
    src = rng.standard_normal((nx, nx, nv, nv))
    vp, vm = nv * (nv + 1) // 2, nv * (nv - 1) // 2
    npr, nmr = nx * (nx + 1) // 2, nx * (nx - 1) // 2
    P, M = np.full((npr, vp), np.nan), np.full((max(nmr, 1), max(vm, 1)), np.nan)
    cnt_p, cnt_m = np.zeros_like(P), np.zeros_like(M)
    nt = (nv + 31) // 32
    h = 0.5
    for bx in range(nt * (nt + 1) // 2):
        F = 0
        while (F + 1) * (F + 2) // 2 <= bx:
            F += 1
        E = bx - F * (F + 1) // 2
        for R in range(npr):
            y = int((np.sqrt(np.float32(8.0 * R + 1.0)) - 1.0) * 0.5)
            while (y + 1) * (y + 2) // 2 <= R:
                y += 1
            while y * (y + 1) // 2 > R:
                y -= 1
            x = R - y * (y + 1) // 2
            t = src[x, y]
            for c in range(32):
                for tx in range(32):
                    f, e = F * 32 + c, E * 32 + tx
                    if f >= nv or e > f:
                        continue
                    a, b = t[e, f], t[f, e]
                    P[R, f * (f + 1) // 2 + e] = a if e == f else h * (a + b)
                    cnt_p[R, f * (f + 1) // 2 + e] += 1
                    if x < y and e < f:
                        M[y * (y - 1) // 2 + x, f * (f - 1) // 2 + e] = h * (a - b)
                        cnt_m[y * (y - 1) // 2 + x, f * (f - 1) // 2 + e] += 1
    assert np.all(cnt_p == 1)
    if nmr and vm:
        assert np.all(cnt_m == 1)
    for y in range(nx):
        for x in range(y + 1):
            for f in range(nv):
                for e in range(f + 1):
                    want = src[x, y, e, e] if e == f else h * (src[x, y, e, f] + src[x, y, f, e])
                    assert P[y * (y + 1) // 2 + x, f * (f + 1) // 2 + e] == want
