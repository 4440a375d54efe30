// gopf_sweep.cpp -- sharding a parameter sweep over processes, one per GPU.
//
// gopf's sweep workflow runs one pf.Solver per parameter set, one after the
// other in one process (README.md:21-33, with one FieldDB per swept run,
// pf/database.go:67-80).  Sweep instances are independent, so a sweep over
// several GPUs needs no exchange at all: each process steps its own share of
// the instances as one batch (gopf_batch_*) and the per-instance results are
// merged on the host afterwards.  This file decides the shares.
//
// The work of an instance per step is proportional to its cell count (every
// pass moves a fixed number of bytes per spectral element), so the shares are
// balanced on cells by greedy longest-processing-time bin packing: instances
// in decreasing cell count (ties: lower index first) each go to the rank
// holding the fewest cells so far (ties: lower rank).  The result depends only
// on the cell counts and the number of ranks, so every process computes the
// same partition without communicating, and every instance has exactly one
// owner.
#include <algorithm>
#include <numeric>
#include <vector>

#include "../../include/gopf_gpu.h"

extern "C" int gopf_sweep_partition(const long long *cells, int n, int world, int *owner, long long *rank_cells)
{
    if (n < 0 || world < 1 || (n > 0 && (!cells || !owner))) return GOPF_ERR_ARG;
    for (int i = 0; i < n; ++i)
        if (cells[i] < 0) return GOPF_ERR_ARG;
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cells[a] > cells[b]; });
    std::vector<long long> load(world, 0);
    for (int i : order) {
        int best = 0;
        for (int r = 1; r < world; ++r)
            if (load[r] < load[best]) best = r;
        owner[i] = best;
        load[best] += cells[i];
    }
    if (rank_cells)
        for (int r = 0; r < world; ++r) rank_cells[r] = load[r];
    return GOPF_OK;
}
