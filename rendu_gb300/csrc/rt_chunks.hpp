// Chunk plan of the pipelined host-buffer path (rt_api.cu): how n records are cut into the
// chunks that are copied in, traversed and copied out. Host-only, no CUDA.
#pragma once

#include <algorithm>
#include <cstddef>
#include <vector>

namespace rgb {

// Chunk sizes for n records: at most `chunk` each, the last three halving (chunk / 2,
// chunk / 4, chunk / 8), so that what follows the last copy-in (that chunk's traversal and
// copy-out) is short. Smaller chunks elsewhere only add launches: a traversal launch lasts
// at least the latency of its longest rays, about 0.15 ms whatever its size. Inputs too
// small for the tail (fewer than 2 chunks + the tail) are cut into equal-size chunks but
// the last.
inline std::vector<size_t> chunk_plan(size_t n, size_t chunk) {
    const size_t tail[3] = {chunk / 2, chunk / 4, chunk / 8};
    const size_t tsum = tail[0] + tail[1] + tail[2];
    std::vector<size_t> v;
    if (n < tsum + 2 * chunk) {
        for (size_t s = 0; s < n; s += chunk) v.push_back(std::min(chunk, n - s));
        return v;
    }
    const size_t mid = n - tsum, k = (mid + chunk - 1) / chunk;
    for (size_t i = 0; i < k; ++i) v.push_back(mid / k + (i < mid % k ? 1 : 0));
    v.insert(v.end(), tail, tail + 3);
    return v;
}

}  // namespace rgb
