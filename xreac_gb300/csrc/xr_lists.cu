// Caller-supplied neighbour lists: validation with xreac's rules and canonical order (host only).
//
// xreac validates a supplied list in Neighbors.__init__ (src/xreac/neighbors.py:104-121) and sorts it
// with packed integer keys in _edge_order (src/xreac/neighbors.py:65-98), raising ValueError for
// duplicates and for edges without their reverse. Here the list is bucketed by source atom (a
// counting pass, O(M)) and each row sorted on a packed key of two 64-bit words (j, Sx, Sy, Sz) with
// the shifts biased into 20-bit fields, so a row of a few hundred edges sorts in cache; duplicates are then
// adjacent, and the reverse of (i, j, S) is found by binary search for (i, -S) in row j.
#include <algorithm>
#include <climits>
#include <cstdint>
#include <cstdlib>

#include "xr_common.cuh"
#include "xr_lists.h"

namespace {

constexpr int kBias = 1 << 19;  // shift field bias: shifts within +-(2^19 - 1) pack exactly

// Key of (j, S) within a row: j and three 20-bit biased shifts need 86 bits, so the key is two words
// compared lexicographically, which is the (j, Sx, Sy, Sz) order.
struct Key {
  uint64_t hi;  // j << 20 | (Sx + bias)
  uint64_t lo;  // (Sy + bias) << 20 | (Sz + bias)
  bool operator<(const Key& o) const { return hi < o.hi || (hi == o.hi && lo < o.lo); }
  bool operator==(const Key& o) const { return hi == o.hi && lo == o.lo; }
};

inline Key make_key(int j, int sx, int sy, int sz) {
  return Key{((uint64_t)(uint32_t)j << 20) | (uint64_t)(uint32_t)(sx + kBias),
             ((uint64_t)(uint32_t)(sy + kBias) << 20) | (uint64_t)(uint32_t)(sz + kBias)};
}

}  // namespace

namespace xr_host {

int canonical_list(int natoms, const int pbc[3], const xr_neighbors& nb, std::vector<int>& start,
                   std::vector<int2>& rows, int maxs[3], std::string& err) {
  const long long m = nb.count;
  if (m < 0 || natoms < 1 || (m > 0 && (!nb.i || !nb.j || !nb.S))) {
    err = "neighbors require i and j with shape (M,) and S with shape (M, 3)";
    return XR_EINPUT;
  }
  if (m > (1ll << 31) - 2) {
    err = "A neighbor list of more than 2^31 - 2 edges is not supported";
    return XR_ECAPACITY;
  }
  const int* I = nb.i;
  const int* J = nb.j;
  const int* S = nb.S;
  for (long long e = 0; e < m; ++e)
    if (I[e] < 0 || J[e] < 0 || I[e] >= natoms || J[e] >= natoms) {
      err = "Neighbor atom indices are out of range";
      return XR_EINPUT;
    }
  for (long long e = 0; e < m; ++e)
    for (int k = 0; k < 3; ++k)
      if (!pbc[k] && S[3 * e + k] != 0) {
        err = "Neighbor shifts must be zero in nonperiodic directions";
        return XR_EINPUT;
      }
  for (long long e = 0; e < m; ++e)
    if (I[e] == J[e] && S[3 * e] == 0 && S[3 * e + 1] == 0 && S[3 * e + 2] == 0) {
      err = "Zero-shift self neighbors are not allowed";
      return XR_EINPUT;
    }
  // Shifts beyond the key's fields cannot be ordered here; they are also far beyond what the device
  // code holds, so such a list is rejected as a capacity error.
  maxs[0] = maxs[1] = maxs[2] = 0;
  bool wide = false;
  for (long long e = 0; e < 3 * m; ++e) {
    const int a = std::abs(S[e] == INT32_MIN ? INT32_MAX : S[e]);
    maxs[e % 3] = std::max(maxs[e % 3], a);
    wide = wide || a >= kBias;
  }
  if (wide) {
    err = "An image shift exceeds the supported range of +-255 cells; wrap the positions into the cell";
    return XR_ECAPACITY;
  }
  // bucket by source atom, then sort each row on its keys
  start.assign((size_t)natoms + 1, 0);
  for (long long e = 0; e < m; ++e) ++start[(size_t)I[e] + 1];
  for (int a = 0; a < natoms; ++a) start[a + 1] += start[a];
  std::vector<Key> keys((size_t)m);
  {
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (long long e = 0; e < m; ++e) keys[fill[I[e]]++] = make_key(J[e], S[3 * e], S[3 * e + 1], S[3 * e + 2]);
  }
  for (int a = 0; a < natoms; ++a) std::sort(keys.begin() + start[a], keys.begin() + start[a + 1]);
  for (int a = 0; a < natoms; ++a)
    for (int e = start[a] + 1; e < start[a + 1]; ++e)
      if (keys[e] == keys[e - 1]) {
        err = "Duplicate neighbor edges are not allowed";
        return XR_EINPUT;
      }
  auto field = [](uint64_t v) { return (int)(v & ((1u << 20) - 1)) - kBias; };
  for (int a = 0; a < natoms; ++a)
    for (int e = start[a]; e < start[a + 1]; ++e) {
      const Key& k = keys[e];
      const int j = (int)(k.hi >> 20), sx = field(k.hi), sy = field(k.lo >> 20), sz = field(k.lo);
      const Key want = make_key(a, -sx, -sy, -sz);
      if (!std::binary_search(keys.begin() + start[j], keys.begin() + start[j + 1], want)) {
        err = "neighbors must include both directions: (i, j, S) and (j, i, -S)";
        return XR_EINPUT;
      }
    }
  if (maxs[0] > XR_SHIFT_MAX || maxs[1] > XR_SHIFT_MAX || maxs[2] > XR_SHIFT_MAX) {
    err = "An image shift exceeds the supported range of +-255 cells; wrap the positions into the cell";
    return XR_ECAPACITY;
  }
  rows.resize((size_t)m);
  for (long long e = 0; e < m; ++e) {
    const Key& k = keys[e];
    rows[e] = make_int2((int)(k.hi >> 20), (int)xr_pack_shift(field(k.hi), field(k.lo >> 20), field(k.lo)));
  }
  return XR_OK;
}

}  // namespace xr_host

extern "C" int xr_neighbors_check(int natoms, const int* pbc, const xr_neighbors* nb, char* msg, int msg_len) {
  std::vector<int> start;
  std::vector<int2> rows;
  int maxs[3];
  std::string err;
  const int flags[3] = {pbc ? pbc[0] : 0, pbc ? pbc[1] : 0, pbc ? pbc[2] : 0};
  int code = XR_EINPUT;
  if (!nb) {
    err = "neighbors must be a tuple (i, j, S)";
  } else {
    code = xr_host::canonical_list(natoms, flags, *nb, start, rows, maxs, err);
  }
  if (msg && msg_len > 0) {
    const size_t n = std::min<size_t>(err.size(), (size_t)msg_len - 1);
    std::copy(err.begin(), err.begin() + n, msg);
    msg[n] = '\0';
  }
  return code;
}
