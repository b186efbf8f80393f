"""Index arithmetic of the symmetric layout, checked on the CPU (no GPU).

The symmetric kernels (single system, compensated, FP64, adjoint, batched)
share one work layout: row blocks of rb bodies paired with the 32-body chunks
at or after their start, (row, chunk) items split stream-K over persistent
CTAs, target-side partials in slot cta + row, and reactions in a triangular
source-side array.  These tests restate the formulas of nb_internal.cuh
(sym_prefix, sym_soff, sym_row_of, sk_start, sk_owner) and check, for many
sizes, that every index the kernels and integrators compute is in range and
that no two writers share an entry.
"""
import numpy as np
import pytest


def sym_prefix(I, nc, rc):
    return I * nc - rc * (I * (I - 1) // 2)


def sym_soff(r, n, rb):
    return r * n - rb * (r * (r + 1) // 2)


def sym_row_of(it, nc, rc, nrb):
    lo, hi = 0, nrb
    while hi - lo > 1:
        mid = (lo + hi) >> 1
        if sym_prefix(mid, nc, rc) <= it:
            lo = mid
        else:
            hi = mid
    return lo


def sk_start(c, total, grid):
    return (c * total) // grid


def sk_owner(it, total, grid):
    return ((it + 1) * grid - 1) // total


def spart_entries(n, rb):
    nrb = -(-n // rb)
    return sym_soff(nrb - 1, n, rb) if nrb > 1 else 0


@pytest.mark.parametrize("n,rb,grid", [
    (1, 512, 1216), (31, 512, 1216), (512, 512, 8), (513, 512, 1216), (1000, 256, 7),
    (4097, 384, 300), (9000, 512, 1216), (20000, 2560, 304), (65536, 512, 1216), (70001, 640, 999),
    (1000, 64, 2432), (4097, 128, 1216), (16384, 64, 2432), (3001, 1024, 152), (9000, 2048, 152),
])
def test_symmetric_layout(n, rb, grid):
    rc = rb // 32
    nc = -(-n // 32)
    nrb = -(-n // rb)
    total = sym_prefix(nrb, nc, rc)
    grid = min(grid, total)
    size = spart_entries(n, rb)
    slots = grid + nrb - 1

    # every item belongs to exactly one CTA; rows are found by binary search
    covered = np.zeros(total, np.int64)
    tslot = {}
    spart_writer = np.full(max(size, 1), -1, np.int64)
    for c in range(grid):
        it, end = sk_start(c, total, grid), sk_start(c + 1, total, grid)
        covered[it:end] += 1
        while it < end:
            I = sym_row_of(it, nc, rc, nrb)
            assert sym_prefix(I, nc, rc) <= it < sym_prefix(I + 1, nc, rc)
            rend = sym_prefix(I + 1, nc, rc)
            seg_end = min(end, rend)
            kc0 = I * rc + (it - sym_prefix(I, nc, rc))
            kc1 = I * rc + (seg_end - sym_prefix(I, nc, rc))
            assert I * rc <= kc0 < kc1 <= nc
            # target-side slot of (cta, row): distinct and inside the array
            slot = c + I
            assert slot not in tslot and 0 <= slot < slots
            tslot[slot] = (c, I)
            for kc in range(kc0, kc1):
                if kc < (I + 1) * rc:
                    continue  # chunk inside the own row block: no reaction
                for lane in range(32):
                    j = kc * 32 + lane
                    if j >= n:
                        continue
                    e = sym_soff(I, n, rb) + (j - (I + 1) * rb)
                    assert 0 <= e < size
                    assert spart_writer[e] == -1, "two items write one source-side entry"
                    spart_writer[e] = I * nc + kc
            it = seg_end
    assert (covered == 1).all()

    # the integrator reads, for body i: slots c0..c1 of its row (exactly the
    # CTAs that wrote one) and one source-side entry per earlier row, found
    # by the incremental offset walk; together these are every entry written
    written = set(np.flatnonzero(spart_writer >= 0).tolist())
    read = set()
    for i in range(n):
        I = i // rb
        c0 = sk_owner(sym_prefix(I, nc, rc), total, grid)
        c1 = sk_owner(sym_prefix(I + 1, nc, rc) - 1, total, grid)
        writers = sorted(c for (c, r) in tslot.values() if r == I)
        assert writers == list(range(c0, c1 + 1))
        off = i - rb
        for r in range(I):
            assert off == sym_soff(r, n, rb) + i - (r + 1) * rb
            assert spart_writer[off] // nc == r  # written by an item of row r
            read.add(off)
            off += n - (r + 2) * rb
    assert read == written


@pytest.mark.parametrize("sizes,rb", [([1, 2, 3], 128), ([128, 300, 4097, 1], 384), ([700] * 5, 256),
                                      ([16384, 128, 5000], 512)])
def test_batched_symmetric_layout(sizes, rb):
    """The batched kernels concatenate the systems' items, rows and
    source-side arrays: every system's entries stay inside its own range."""
    rc = rb // 32
    it_off, row_off, sp_off = [0], [0], [0]
    for n in sizes:
        nc, nrb = -(-n // 32), -(-n // rb)
        it_off.append(it_off[-1] + sym_prefix(nrb, nc, rc))
        row_off.append(row_off[-1] + nrb)
        sp_off.append(sp_off[-1] + spart_entries(n, rb))
    for s, n in enumerate(sizes):
        nc, nrb = -(-n // 32), -(-n // rb)
        for I in range(nrb):
            for kc in range(I * rc, nc):
                if kc < (I + 1) * rc:
                    continue
                for j in range(kc * 32, min(kc * 32 + 32, n)):
                    e = sp_off[s] + sym_soff(I, n, rb) + (j - (I + 1) * rb)
                    assert sp_off[s] <= e < sp_off[s + 1]
        assert row_off[s + 1] - row_off[s] == nrb
        assert it_off[s + 1] - it_off[s] == sym_prefix(nrb, nc, rc)
