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
// Compact variant: ring chunks of its factorization, the reload entry's slot
// in its elimination stream, and the flag of a solve entry whose operand is in
// global memory.
constexpr int kCompactRing = 2;
constexpr uint32_t kReloadSlot = 0x7ffeu;
constexpr int32_t kGlobalOperand = 0x40000000;
// The no-op entry's y of the solve streams.
constexpr int32_t kNoop = -2147483647 - 1;

}  // namespace fo
