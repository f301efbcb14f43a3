// Host side of the upwind-sweep plan: the level order of one direction's
// upwind graph.  Plain C++ (no CUDA), so it is also compiled into host tests.
#pragma once

#include <algorithm>
#include <cstdint>
#include <functional>
#include <queue>
#include <utility>
#include <vector>

namespace bte {

inline int inflow_count(uint8_t m) {
    int k = 0;
    for (; m; m >>= 1) k += m & 1;
    return k;
}

// Level order of one direction's upwind graph (Kahn's algorithm in waves).
// mask[c] bit f: face f of c is an inflow face with a neighbour.  When no cell
// is free the unprocessed cell with the fewest unresolved inflow edges (lowest
// index on ties) starts the next level alone and those edges become lagged.
// That cell is found in a min-heap of (unresolved inflow edges, cell), built at
// the first such break and kept current lazily (a decrement pushes a new entry;
// stale entries are skipped), so a graph with many cycles costs O(n log n),
// not O(n) per break; acyclic graphs never build it.
inline void level_order(int n, int F, const uint8_t* mask, const int* nbr, std::vector<int>& perm,
                        std::vector<int>& lvl, std::vector<int>& lagged /* [F][n] */) {
    std::vector<int> indeg(n), dptr(n + 1, 0), down;
    for (int c = 0; c < n; ++c) {
        int k = 0;
        for (int f = 0; f < F; ++f)
            if (mask[c] >> f & 1) { ++k; ++dptr[nbr[(size_t)c * F + f] + 1]; }
        indeg[c] = k;
    }
    for (int c = 0; c < n; ++c) dptr[c + 1] += dptr[c];
    down.resize(dptr[n]);
    std::vector<int> fill(dptr.begin(), dptr.end() - 1);
    for (int c = 0; c < n; ++c)
        for (int f = 0; f < F; ++f)
            if (mask[c] >> f & 1) down[fill[nbr[(size_t)c * F + f]]++] = c;
    std::vector<char> done(n, 0);
    std::vector<int> wave, next;
    for (int c = 0; c < n; ++c)
        if (indeg[c] == 0) wave.push_back(c);
    perm.clear();
    lvl.clear();
    lagged.assign((size_t)F * n, 0);
    using Entry = std::pair<int, int>;  // (unresolved inflow edges, cell)
    std::priority_queue<Entry, std::vector<Entry>, std::greater<Entry>> heap;
    bool heap_on = false;
    int processed = 0;
    while (processed < n) {
        if (wave.empty()) {
            if (!heap_on) {
                for (int c = 0; c < n; ++c)
                    if (!done[c]) heap.push({indeg[c], c});
                heap_on = true;
            }
            int best = -1;
            while (best < 0) {
                const Entry top = heap.top();
                heap.pop();
                if (!done[top.second] && indeg[top.second] == top.first) best = top.second;
            }
            for (int f = 0; f < F; ++f)
                if ((mask[best] >> f & 1) && !done[nbr[(size_t)best * F + f]]) lagged[(size_t)f * n + best] = 1;
            wave.push_back(best);
        }
        std::sort(wave.begin(), wave.end());
        lvl.push_back((int)perm.size());
        for (int c : wave) { done[c] = 1; perm.push_back(c); }
        processed += (int)wave.size();
        next.clear();
        for (int c : wave)
            for (int k = dptr[c]; k < dptr[c + 1]; ++k) {
                const int c2 = down[k];
                if (done[c2]) continue;
                if (--indeg[c2] == 0) next.push_back(c2);
                else if (heap_on) heap.push({indeg[c2], c2});
            }
        wave.swap(next);
    }
    lvl.push_back(n);
}

}  // namespace bte
