// Host side of caller-supplied neighbour lists (xr_eval_neighbors, xr_neighbors_check).
#pragma once
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "xreac_gb300.h"

namespace xr_host {

// Validates a directed list (i, j, S) of a system of `natoms` atoms with xreac's rules, in xreac's
// order (src/xreac/neighbors.py:104-121 and _edge_order, 65-98): indices in range, zero shifts in
// non-periodic directions, no zero-shift self edge, no duplicate edge, both directions present.
// On success fills `start` (natoms + 1 row offsets) and `rows` ({j, packed shift bits} per edge, each
// row in canonical (j, Sx, Sy, Sz) order) and maxs[k] = the largest |S_k|. Returns XR_OK, XR_EINPUT
// with xreac's message in `err`, or XR_ECAPACITY when a valid list has a shift beyond +-255 cells
// (the device's packed edge code).
int canonical_list(int natoms, const int pbc[3], const xr_neighbors& nb, std::vector<int>& start,
                   std::vector<int2>& rows, int maxs[3], std::string& err);

}  // namespace xr_host
