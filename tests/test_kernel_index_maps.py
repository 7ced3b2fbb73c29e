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
