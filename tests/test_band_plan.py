"""The band partition of the symmetric kernels' triangular source side
(nb::sym_make_bands), checked on the host: the probe in
tests/band_plan_probe.cu is built from the library's own header and run for
sizes up to N = 2^30 (no GPU)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CAP8 = (8 << 30) // 16  # the 8 GiB budget in float4 entries


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    out = str(tmp_path_factory.mktemp("bands") / "band_plan_probe")
    subprocess.run([nvcc, "-O1", "-std=c++17", "-I", os.path.join(REPO, "include"), "-I",
                    os.path.join(REPO, "utc_gb300", "csrc"), os.path.join(HERE, "band_plan_probe.cu"), "-o", out],
                   check=True, capture_output=True)

    def run(n, rb, cap, want):
        f = subprocess.run([out, str(n), str(rb), str(cap), str(want)], check=True, capture_output=True,
                           text=True).stdout.split()
        k, mx, total = int(f[0]), int(f[1]), int(f[2])
        return k, mx, total, [int(x) for x in f[3:]]
    return run


def entries(n, rb, r0, r1):
    nrb = -(-n // rb)
    return sum(n - (r + 1) * rb for r in range(r0, min(r1, nrb - 1)))


CASES = [(4096, 512), (65536, 512), (262144, 512), (1048576, 2560), (1700000, 2560), (2097152, 2560),
         (6000000, 2560), (300000, 64), (1048576, 64), (1 << 30, 2560), (1000, 128), (1, 512)]


@pytest.mark.parametrize("n,rb", CASES)
def test_bands_cover_rows_within_the_budget(probe, n, rb):
    """Automatic bands: consecutive row blocks from 0 to nrb, each band's
    entries within the cap unless it is a single row, each boundary forced
    (the next row would have passed the cap), entries summing to the
    triangular array's; beyond 512 bands the plan refuses (0)."""
    nrb = -(-n // rb)
    k, mx, total, rows = probe(n, rb, CAP8, 0)
    assert total == entries(n, rb, 0, nrb)
    if k == 0:
        assert total > 511 * CAP8  # more than the plan holds
        return
    assert rows[0] == 0 and rows[-1] == nrb and len(rows) == k + 1
    assert all(a < b for a, b in zip(rows, rows[1:]))
    sizes = [entries(n, rb, a, b) for a, b in zip(rows, rows[1:])]
    assert sum(sizes) == total and max(sizes) == mx
    for (a, b), e in zip(zip(rows, rows[1:]), sizes):
        assert e <= CAP8 or b - a == 1
    for (a, b), (_, c) in zip(zip(rows, rows[1:]), zip(rows[1:], rows[2:])):
        assert entries(n, rb, a, b + 1) > CAP8  # the boundary at b was needed


@pytest.mark.parametrize("n,rb", [c for c in CASES if c[0] <= 6000000 and c[0] > 1])
@pytest.mark.parametrize("want", [2, 3, 7, 64, 512])
def test_requested_bands(probe, n, rb, want):
    """nb_params.bands = want: a valid partition of at most `want` bands
    (more only where the budget needs more, fewer where there are fewer
    row blocks), and, where there are rows enough to split evenly, bands
    of about equal size (the largest within twice the mean)."""
    nrb = -(-n // rb)
    k, mx, total, rows = probe(n, rb, CAP8, want)
    auto = probe(n, rb, CAP8, 0)[0]
    assert 1 <= k <= max(want, auto) and k <= nrb
    assert rows[0] == 0 and rows[-1] == nrb and all(a < b for a, b in zip(rows, rows[1:]))
    sizes = [entries(n, rb, a, b) for a, b in zip(rows, rows[1:])]
    assert sum(sizes) == total and max(sizes) == mx
    if auto <= want and 4 * want <= nrb:
        assert k >= want // 2
        assert mx <= 2 * total / want
