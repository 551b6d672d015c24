// poe2d_plan.h -- the balanced work-list order of the persistent step kernel
// (host code, no CUDA types).
//
// The step kernel's CTAs take the items of its work list in order, each the
// next one from a shared counter.  Edge tiles (a grid edge, a C-PML strip or
// the source within reach of the tile and its halo) take about twice the work
// of an interior tile and wait on global loads of the C-PML memory; in rows
// order they come in runs (a 2001^2 shot's first two and last two tile rows
// are all edge tiles: 313 of its 2142 tiles), during which every SM is on the
// strips.
//
// balanced_order() spreads them evenly through the list: with `slots`
// positions per round (the SM count), the edge tiles go to the positions a
// water-filling deal of them over the slots gives (so that with one CTA per
// slot each CTA's work, 1 per tile and 1 more per edge tile, is as even as the
// counts allow), each slot's spread evenly over its positions (Bresenham), and
// edge and interior tiles each keep their order, so the tiles that run side
// by side stay neighbours (their halos are shared through L2).  The result is
// a permutation: position p holds item order[p].  Tiles are independent within
// a step, so any order gives the same results bit for bit.
#pragma once
#include <stdint.h>

#include <algorithm>
#include <vector>

namespace poe {

inline std::vector<int> balanced_order(const std::vector<uint8_t> &edge, int slots)
{
    const int n = (int)edge.size();
    std::vector<int> order;
    order.reserve((size_t)n);
    if (n == 0) return order;
    const int S = std::max(1, std::min(slots, n));
    const int q = n / S, r = n % S;                  // CTA b holds q + (b < r) positions
    int E = 0;
    for (uint8_t e : edge) E += e ? 1 : 0;
    auto npos = [&](int b) { return q + (b < r ? 1 : 0); };
    // smallest level L (work of the busiest CTA) whose edge capacity, sum over
    // CTAs of min(npos, L - npos), holds every edge tile
    auto capacity = [&](int L) {
        int64_t c = 0;
        for (int b = 0; b < S; ++b) c += std::max(0, std::min(npos(b), L - npos(b)));
        return c;
    };
    int L = q;
    while (capacity(L) < E) ++L;                     // L <= 2 (q + 1): every position an edge tile
    std::vector<int> quota((size_t)S);
    int64_t excess = -E;
    for (int b = 0; b < S; ++b) {
        quota[(size_t)b] = std::max(0, std::min(npos(b), L - npos(b)));
        excess += quota[(size_t)b];
    }
    // give back the surplus, first from the CTAs at the level, then from any
    for (int pass = 0; pass < 2 && excess > 0; ++pass)
        for (int b = S - 1; b >= 0 && excess > 0; --b)
            if (quota[(size_t)b] > 0 && (pass == 1 || npos(b) + quota[(size_t)b] == L)) {
                --quota[(size_t)b];
                --excess;
            }
    std::vector<int> edges, inner;
    for (int i = 0; i < n; ++i) (edge[(size_t)i] ? edges : inner).push_back(i);
    size_t ne = 0, ni = 0;
    for (int p = 0; p < n; ++p) {
        const int b = p % S, k = p / S;
        const int64_t nb = npos(b), eb = quota[(size_t)b];
        const bool take_edge = (k + 1) * eb / nb > k * eb / nb;   // the k-th of nb positions holds an edge tile
        if ((take_edge && ne < edges.size()) || ni == inner.size()) order.push_back(edges[ne++]);
        else order.push_back(inner[ni++]);
    }
    return order;
}

}  // namespace poe
