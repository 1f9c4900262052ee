// Test driver (CPU): lcg_host::queue_order, the work-queue order of the fill
// and LocARNA-P kernels. stdin: "<pairs> <budget bytes>" then per pair
// "<groups> <bytes>". Prints "ok" when every (pair, group) item appears
// exactly once and each pair's groups keep their own order (group g before
// g + 1: the dependency order of one pair, so that the queue and its reverse
// are valid for the dataflow kernels), then the number of waves the budget
// gave; else "bad <reason>".
#include <cstdio>
#include <iostream>
#include <vector>

#include "../../locarna_gb300/csrc/engine_prep.hh"

int main() {
    int np;
    double budget;
    std::cin >> np >> budget;
    std::vector<size_t> ng(np);
    std::vector<double> by(np);
    size_t total = 0;
    for (int q = 0; q < np; ++q) {
        std::cin >> ng[q] >> by[q];
        total += ng[q];
    }
    std::vector<int2> out(total, make_int2(-1, -1));
    lcg_host::queue_order(
        ng, [&](int q) { return by[q]; }, out.data(), [](int n, auto fn) { lcg_host::parallel_for(n, fn); },
        budget);
    std::vector<long long> next(np, 0);
    int waves = 0, last_first = -1;
    for (size_t k = 0; k < total; ++k) {
        const int q = out[k].x, g = out[k].y;
        if (q < 0 || q >= np) {
            std::printf("bad pair index at %zu\n", k);
            return 0;
        }
        if (g != next[q]) {
            std::printf("bad order: pair %d group %d where %lld was due\n", q, g, next[q]);
            return 0;
        }
        ++next[q];
        if (g == 0 && q > last_first) {
            // a pair's first group: count a new wave when the pairs of an
            // earlier wave are all done
            bool done = true;
            for (int p = 0; p <= last_first && done; ++p) done = next[p] == (long long)ng[p];
            if (done) ++waves;
            last_first = q;
        }
    }
    for (int q = 0; q < np; ++q)
        if (next[q] != (long long)ng[q]) {
            std::printf("bad count for pair %d\n", q);
            return 0;
        }
    std::printf("ok %d\n", waves);
    return 0;
}
