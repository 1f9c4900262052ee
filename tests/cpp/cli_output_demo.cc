// Test driver (CPU): the command lines' alignment writer (lcg_output.hh) on
// given alignment edges. stdin: "<rows A> <rows B> <width> <stockholm 0/1>",
// the rows of A then of B as "name sequence", then "<k>" and k edges "a b"
// (-1 for a gap), optionally followed by "<j>" and j anchor lines of A, then
// "<l>" and l anchor lines of B. Prints the CLUSTAL (or Stockholm) blocks
// with the consensus anchor lines.
#include <iostream>
#include <string>
#include <vector>

#include "../../locarna_gb300/cli/lcg_output.hh"

int main() {
    int na, nb, width, sto;
    std::cin >> na >> nb >> width >> sto;
    std::vector<lcg_cli::Row> a(na), b(nb);
    for (auto &r : a) std::cin >> r.name >> r.seq;
    for (auto &r : b) std::cin >> r.name >> r.seq;
    int k;
    std::cin >> k;
    lcg_cli::Edges raw(k);
    for (auto &e : raw) std::cin >> e.first >> e.second;
    std::vector<std::string> anch_a, anch_b;
    int j = 0, l = 0;
    if (std::cin >> j) {
        anch_a.resize(j);
        for (auto &s : anch_a) std::cin >> s;
        std::cin >> l;
        anch_b.resize(l);
        for (auto &s : anch_b) std::cin >> s;
    }
    const int n = (int)a[0].seq.size(), m = (int)b[0].seq.size();
    const auto edges = lcg_cli::alignment_edges(raw, n, m);
    lcg_cli::write_blocks(std::cout, lcg_cli::rows(edges, a, b), (size_t)width, sto != 0,
                          lcg_cli::anchor_consensus(edges, anch_a, anch_b));
    return 0;
}
