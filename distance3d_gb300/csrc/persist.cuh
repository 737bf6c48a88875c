// persist.cuh -- work distribution for persistent kernels.
//
// Every lane owns one pair at a time and fetches the next as soon as its pair
// finishes, so a warp stays full while work remains instead of waiting for
// its slowest pair.  Fetches are warp-aggregated: one atomic per warp per
// round, slots handed out in lane order (fetch_slot), or one atomic per warp
// per chunk of slots that the warp then hands to its lanes
// (fetch_slot_chunked), which keeps a warp's lanes on neighbouring pairs of a
// sorted order.
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

// A warp's share of the global order: the slots [next, end) it has claimed
// and not yet handed to a lane.  Every lane holds the same copy.
struct WarpChunk {
    long long next = 0, end = 0;
};

// Lanes with `need` set receive consecutive slots (-1 for the others), taken
// from the warp's chunk; when the chunk runs out the warp claims the next
// `chunk` (>= 32) slots of *cursor.  A warp's lanes then hold pairs from at
// most two chunks of the order at a time, instead of from anywhere in the
// span all resident lanes of the GPU have fetched, which keeps the lanes of
// a warp on pairs of the same collider types in a type-sorted order.  Once
// the cursor has passed `split` (the caller's n minus a few slots per
// resident lane) a warp claims only the slots its lanes ask for, so that no
// slot waits in the chunk of a busy warp at the end of the order.
// Every lane of `live` must call it together (converged), so that the
// lanes' copies of `w` stay equal.
__device__ __forceinline__ long long fetch_slot_chunked(unsigned long long* cursor, bool need, WarpChunk& w,
                                                        unsigned live, int chunk, long long split) {
    const unsigned want = __ballot_sync(live, need);
    if (!want) return -1;
    const int lane = threadIdx.x & 31;
    const int rank = __popc(want & ((1u << lane) - 1u));
    const int cnt = __popc(want);
    const long long avail = w.end - w.next;
    long long slot;
    if (avail >= cnt) {
        slot = w.next + rank;
        w.next += cnt;
    } else {
        const int leader = __ffs(live) - 1;
        unsigned long long base = 0;
        int size = 0;
        if (lane == leader) {
            // the cursor's value is only a hint for the claim's size
            const long long seen = (long long)*reinterpret_cast<volatile unsigned long long*>(cursor);
            size = seen + chunk <= split ? chunk : cnt - (int)avail;
            base = atomicAdd(cursor, (unsigned long long)size);
        }
        base = __shfl_sync(live, base, leader);
        size = __shfl_sync(live, size, leader);
        slot = rank < avail ? w.next + rank : (long long)base + (rank - avail);
        w.next = (long long)base + (cnt - avail);
        w.end = (long long)base + size;
    }
    return need ? slot : -1;
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

// The same for the lanes of `mask`, all of which must call it together.
__device__ __forceinline__ void append_lanes(unsigned mask, int32_t* list, unsigned long long* count, bool take,
                                             int32_t value) {
    const unsigned want = __ballot_sync(mask, take);
    if (!want) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(want) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(count, (unsigned long long)__popc(want));
    base = __shfl_sync(mask, base, leader);
    if (take) list[base + __popc(want & ((1u << lane) - 1u))] = value;
}

}  // namespace d3d
