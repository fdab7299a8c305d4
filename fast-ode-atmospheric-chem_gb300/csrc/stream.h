// Constants shared by the host stream builder and the device kernels.
#pragma once

#include <cstdint>

namespace fo {

// Entries per software-pipelined chunk of the elimination and solve streams.
constexpr int kStreamChunk = 16;
// Chunks of the factorization's shared-memory prefetch ring.
constexpr int kRingChunks = 5;
// Chunks over which the elimination stream is hazard-free (see symbolic.cpp).
constexpr int kHazardWindow = 1;
// The no-op entry's y of the solve streams.
constexpr int32_t kNoop = -2147483647 - 1;

}  // namespace fo
