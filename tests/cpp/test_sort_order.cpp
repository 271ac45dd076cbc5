// Replays opiv::sort_order_head against std::sort on tie-heavy random
// candidate lists: the head it reports must equal std::sort's, element for
// element (keys included), which is what find_peaks' first peak depends on.
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

#include "sort_order.h"

int main()
{
    std::mt19937_64 rng(12345);
    long checked = 0;
    for (int trial = 0; trial < 20000; ++trial) {
        const int n = (int)(rng() % 700);
        const int distinct = 1 + (int)(rng() % 12);
        std::vector<opiv::peak_cand> a(n);
        for (int i = 0; i < n; ++i) a[i] = { (double)(rng() % distinct), i };
        if (trial % 7 == 0)   // sorted / reverse-sorted runs
            std::sort(a.begin(), a.end(), [&](auto& p, auto& q) { return (trial % 2) ? p.v < q.v : p.v > q.v; });
        std::vector<opiv::peak_cand> ref = a, got = a;
        std::sort(ref.begin(), ref.end(), [](const opiv::peak_cand& p, const opiv::peak_cand& q) { return p.v > q.v; });
        const int k = opiv::sort_order_head(got.data(), n);
        if (n > 0 && (k < 1 || k > n)) { std::printf("bad k %d for n %d\n", k, n); return 1; }
        for (int i = 0; i < k; ++i)
            if (got[i].key != ref[i].key || got[i].v != ref[i].v) {
                std::printf("mismatch trial %d n %d at %d\n", trial, n, i);
                return 1;
            }
        checked += k;
    }
    std::printf("ok %ld\n", checked);
    return 0;
}
