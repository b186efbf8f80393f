// Host-only probe of the triangular source side's band partition
// (nb::sym_make_bands in nb_internal.cuh); no device code runs.  Used by
// tests/test_band_plan.py.
//   band_plan_probe n rb cap want
// prints: bands  largest_band_entries  total_entries  row_0 ... row_bands
#include <cstdio>
#include <cstdlib>

#include "nb_internal.cuh"

int main(int argc, char **argv)
{
    if (argc != 5) return 2;
    const int n = atoi(argv[1]), rb = atoi(argv[2]);
    const long long cap = atoll(argv[3]);
    const int want = atoi(argv[4]);
    static int rows[nb::SymPlan::kMaxBands + 1];
    long long mx = 0;
    const int k = nb::sym_make_bands(n, rb, cap, want, rows, &mx);
    printf("%d %lld %lld", k, mx, nb::sym_spart_entries(n, rb));
    for (int b = 0; k > 0 && b <= k; ++b) printf(" %d", rows[b]);
    printf("\n");
    return 0;
}
