// persist.cuh -- work distribution for persistent kernels.
//
// Every lane owns one pair at a time and fetches the next as soon as its pair
// finishes, so a warp stays full while work remains instead of waiting for
// its slowest pair.  Fetches are warp-aggregated: one atomic per warp per
// round, slots handed out in lane order.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace d3d {

// Lanes with `need` set receive consecutive slots from *cursor (-1 for the
// others).  Must be called by every active lane of the warp.
__device__ __forceinline__ long long fetch_slot(unsigned long long* cursor, bool need) {
    const unsigned active = __activemask();
    const unsigned want = __ballot_sync(active, need);
    long long slot = -1;
    if (want) {
        const int lane = threadIdx.x & 31;
        const int leader = __ffs(want) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(cursor, (unsigned long long)__popc(want));
        base = __shfl_sync(active, base, leader);
        if (need) slot = (long long)(base + __popc(want & ((1u << lane) - 1u)));
    }
    return slot;
}

// Lanes with `take` set append `value` to list[*count ...], one atomic per
// warp, in lane order.  Must be called by every active lane of the warp.
__device__ __forceinline__ void append_warp(int32_t* list, unsigned long long* count, bool take, int32_t value) {
    const unsigned active = __activemask();
    const unsigned want = __ballot_sync(active, take);
    if (!want) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(want) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(count, (unsigned long long)__popc(want));
    base = __shfl_sync(active, base, leader);
    if (take) list[base + __popc(want & ((1u << lane) - 1u))] = value;
}

}  // namespace d3d
