// bvh.cu -- broad phase: a linear BVH over FP64 axis-aligned boxes.
//
// Build (all on the device):
//   1. bounds of the box centers (block reduction + one-block reduction);
//   2. 63-bit Morton codes of the centers (21 bits per axis), radix-sorted
//      with the leaf index as payload (CUB);
//   3. Karras' (2012) parallel hierarchy: one thread per internal node finds
//      its key range and split from common-prefix lengths, equal codes tied
//      by index;
//   4. bottom-up refit with one atomic visit counter per internal node (no
//      waiting: the second child to arrive merges and climbs on).
// Internal node boxes are FP32 rounded outward (lower bounds down, upper
// bounds up), so a box that overlaps in FP64 also overlaps in FP32: pruning
// never loses a pair.  Leaves are tested with the caller's exact FP64 boxes
// and the reference's closed-interval rule (aabb_tree.py:504-527), so the
// pair sets equal the reference's AabbTree / brute-force sets bit for bit.
//
// Queries walk the tree with a per-thread stack and compact hits with a warp
// ballot (one atomic per warp and round).  Hits are 64-bit keys sorted on the
// device, so the output order is fixed: self pairs (i, j), i < j ascending;
// box queries (leaf, query) ascending.
#include <cub/cub.cuh>

#include "capi_util.h"
#include "scratch.h"

namespace {

constexpr int kBlock = 256;
constexpr int kStack = 128;
constexpr int kBoundBlocks = 512;

inline size_t up(size_t x) { return (x + 255) & ~size_t(255); }

// ----------------------------------------------------------- tree layout
// All arrays live in one caller-provided buffer; offsets depend on n only.
struct Tree {
    int64_t n;
    int32_t* sorted;    // [n]   sorted position -> original index
    int2* child;        // [n-1] children: c >= 0 internal node, c < 0 leaf ~c (sorted position)
    int2* range;        // [n-1] first/last sorted position under the node
    float4* box;        // [2(n-1)] internal boxes: lo (xyz), hi (xyz), FP32 outward
    float4* leafbox;    // [2n]  leaf boxes in sorted order, FP32 outward
    int32_t* parent;    // [n-1 + n] parents of internal nodes, then of leaves
    int32_t* visits;    // [n-1] refit counters
    uint64_t* keys;     // [n]
    uint64_t* keys_out; // [n]
    int32_t* vals;      // [n]
    double* bounds;     // [2 * 3 * kBoundBlocks + 6]
    int32_t* flags;     // [4] error flags
    void* cub_temp;
    size_t cub_bytes;
};

size_t cub_sort_bytes(int64_t n) {
    size_t b = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, b, (const uint64_t*)nullptr, (uint64_t*)nullptr,
                                    (const int32_t*)nullptr, (int32_t*)nullptr, (int)n, 0, 63);
    return b;
}

size_t layout(void* base, int64_t n, Tree* t) {
    const int64_t ni = n > 1 ? n - 1 : 1;
    const size_t cub_bytes = cub_sort_bytes(n > 0 ? n : 1);
    size_t off = 256;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += up(bytes);
        return o;
    };
    size_t o_sorted = take(sizeof(int32_t) * n);
    size_t o_child = take(sizeof(int2) * ni);
    size_t o_range = take(sizeof(int2) * ni);
    size_t o_box = take(sizeof(float4) * 2 * ni);
    size_t o_leafbox = take(sizeof(float4) * 2 * n);
    size_t o_parent = take(sizeof(int32_t) * (ni + n));
    size_t o_visits = take(sizeof(int32_t) * ni);
    size_t o_keys = take(sizeof(uint64_t) * n);
    size_t o_keys_out = take(sizeof(uint64_t) * n);
    size_t o_vals = take(sizeof(int32_t) * n);
    size_t o_bounds = take(sizeof(double) * (6 * kBoundBlocks + 6));
    size_t o_flags = take(sizeof(int32_t) * 4);
    size_t o_cub = take(cub_bytes);
    if (t) {
        char* b = static_cast<char*>(base);
        t->n = n;
        t->sorted = reinterpret_cast<int32_t*>(b + o_sorted);
        t->child = reinterpret_cast<int2*>(b + o_child);
        t->range = reinterpret_cast<int2*>(b + o_range);
        t->box = reinterpret_cast<float4*>(b + o_box);
        t->leafbox = reinterpret_cast<float4*>(b + o_leafbox);
        t->parent = reinterpret_cast<int32_t*>(b + o_parent);
        t->visits = reinterpret_cast<int32_t*>(b + o_visits);
        t->keys = reinterpret_cast<uint64_t*>(b + o_keys);
        t->keys_out = reinterpret_cast<uint64_t*>(b + o_keys_out);
        t->vals = reinterpret_cast<int32_t*>(b + o_vals);
        t->bounds = reinterpret_cast<double*>(b + o_bounds);
        t->flags = reinterpret_cast<int32_t*>(b + o_flags);
        t->cub_temp = b + o_cub;
        t->cub_bytes = cub_bytes;
    }
    return off;
}

// ----------------------------------------------------------- build kernels
__device__ __forceinline__ void load_box(const double* aabbs, int64_t i, double* lo, double* hi) {
    const double* a = aabbs + 6 * i;  // [axis][min,max]
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = a[2 * k];
        hi[k] = a[2 * k + 1];
    }
}

__global__ void k_center_bounds(const double* __restrict__ aabbs, int64_t n, double* __restrict__ partial) {
    __shared__ double s[6][kBlock];
    double m[6] = {DBL_MAX, DBL_MAX, DBL_MAX, -DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double lo[3], hi[3];
        load_box(aabbs, i, lo, hi);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double c = 0.5 * (lo[k] + hi[k]);
            m[k] = fmin(m[k], c);
            m[3 + k] = fmax(m[3 + k], c);
        }
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) s[k][threadIdx.x] = m[k];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                s[k][threadIdx.x] = fmin(s[k][threadIdx.x], s[k][threadIdx.x + w]);
                s[3 + k][threadIdx.x] = fmax(s[3 + k][threadIdx.x], s[3 + k][threadIdx.x + w]);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 6; ++k) partial[6 * blockIdx.x + k] = s[k][0];
}

__global__ void k_reduce_bounds(double* __restrict__ partial, int blocks, double* __restrict__ out) {
    if (threadIdx.x != 0) return;
    double m[6] = {DBL_MAX, DBL_MAX, DBL_MAX, -DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (int b = 0; b < blocks; ++b)
        for (int k = 0; k < 3; ++k) {
            m[k] = fmin(m[k], partial[6 * b + k]);
            m[3 + k] = fmax(m[3 + k], partial[6 * b + 3 + k]);
        }
    for (int k = 0; k < 6; ++k) out[k] = m[k];
}

__device__ __forceinline__ uint64_t spread21(uint64_t v) {
    v &= 0x1fffff;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

__global__ void k_morton(const double* __restrict__ aabbs, int64_t n, const double* __restrict__ bounds,
                         uint64_t* __restrict__ keys, int32_t* __restrict__ vals) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double lo[3], hi[3];
    load_box(aabbs, i, lo, hi);
    uint64_t q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double ext = bounds[3 + k] - bounds[k];
        double u = ext > 0.0 ? (0.5 * (lo[k] + hi[k]) - bounds[k]) / ext : 0.0;
        double x = u * 2097152.0;
        q[k] = (x != x || x <= 0.0) ? 0ull : (x >= 2097151.0 ? 2097151ull : (uint64_t)x);
    }
    keys[i] = (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
    vals[i] = (int32_t)i;
}

__global__ void k_leaf_boxes(const double* __restrict__ aabbs, int64_t n, const int32_t* __restrict__ sorted,
                             float4* __restrict__ leafbox) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    double lo[3], hi[3];
    load_box(aabbs, sorted[p], lo, hi);
    leafbox[2 * p] = make_float4(__double2float_rd(lo[0]), __double2float_rd(lo[1]), __double2float_rd(lo[2]), 0.f);
    leafbox[2 * p + 1] =
        make_float4(__double2float_ru(hi[0]), __double2float_ru(hi[1]), __double2float_ru(hi[2]), 0.f);
}

// common-prefix length of sorted keys i and j, ties broken by index
__device__ __forceinline__ int delta(const uint64_t* __restrict__ k, int64_t n, int64_t i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    uint64_t a = k[i], b = k[j];
    if (a == b) return 64 + __clz((int)((uint32_t)i ^ (uint32_t)j));
    return __clzll((long long)(a ^ b));
}

__global__ void k_karras(const uint64_t* __restrict__ k, int64_t n, int2* __restrict__ child, int2* __restrict__ range,
                         int32_t* __restrict__ parent) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(k, n, i, i + 1) - delta(k, n, i, i - 1)) > 0 ? 1 : -1;
    const int dmin = delta(k, n, i, i - d);
    int64_t lmax = 2;
    while (delta(k, n, i, i + lmax * d) > dmin) lmax *= 2;
    int64_t l = 0;
    for (int64_t t = lmax / 2; t >= 1; t /= 2)
        if (delta(k, n, i, i + (l + t) * d) > dmin) l += t;
    const int64_t j = i + l * d;
    const int dnode = delta(k, n, i, j);
    int64_t s = 0, t = l;
    do {
        t = (t + 1) / 2;
        if (delta(k, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int64_t gamma = i + s * d + (d < 0 ? -1 : 0);
    const int64_t lo = i < j ? i : j, hi = i < j ? j : i;
    const int left = lo == gamma ? ~(int)gamma : (int)gamma;
    const int right = hi == gamma + 1 ? ~(int)(gamma + 1) : (int)(gamma + 1);
    child[i] = make_int2(left, right);
    range[i] = make_int2((int)lo, (int)hi);
    const int64_t ni = n - 1;
    parent[left >= 0 ? left : ni + ~left] = (int32_t)i;
    parent[right >= 0 ? right : ni + ~right] = (int32_t)i;
}

__device__ __forceinline__ void child_box(const Tree& t, int c, float4& lo, float4& hi) {
    if (c < 0) {
        lo = t.leafbox[2 * (int64_t)~c];
        hi = t.leafbox[2 * (int64_t)~c + 1];
    } else {
        lo = __ldcg(t.box + 2 * (int64_t)c);
        hi = __ldcg(t.box + 2 * (int64_t)c + 1);
    }
}

__global__ void k_refit(Tree t) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= t.n) return;
    const int64_t ni = t.n - 1;
    int node = t.parent[ni + p];
    int guard = 0;
    while (node >= 0 && guard++ < 4 * kStack) {
        __threadfence();
        if (atomicAdd(t.visits + node, 1) == 0) return;  // the sibling subtree is not done yet
        int2 c = t.child[node];
        float4 alo, ahi, blo, bhi;
        child_box(t, c.x, alo, ahi);
        child_box(t, c.y, blo, bhi);
        __stcg(t.box + 2 * (int64_t)node, make_float4(fminf(alo.x, blo.x), fminf(alo.y, blo.y), fminf(alo.z, blo.z), 0.f));
        __stcg(t.box + 2 * (int64_t)node + 1,
               make_float4(fmaxf(ahi.x, bhi.x), fmaxf(ahi.y, bhi.y), fmaxf(ahi.z, bhi.z), 0.f));
        node = t.parent[node];
    }
    if (node >= 0) atomicExch(t.flags, 1);
}

// ----------------------------------------------------------- queries
__device__ __forceinline__ bool overlap32(const float4& alo, const float4& ahi, const float4& blo, const float4& bhi) {
    return alo.x <= bhi.x && ahi.x >= blo.x && alo.y <= bhi.y && ahi.y >= blo.y && alo.z <= bhi.z && ahi.z >= blo.z;
}

// aabb_tree.py:504-527, closed intervals
__device__ __forceinline__ bool overlap64(const double* a, const double* b) {
    return a[0] <= b[1] && a[1] >= b[0] && a[2] <= b[3] && a[3] >= b[2] && a[4] <= b[5] && a[5] >= b[4];
}

// warp-ballot compaction of one hit per lane
__device__ __forceinline__ void emit(bool want, uint64_t key, unsigned long long* count, uint64_t* out,
                                     int64_t cap) {
    const unsigned active = __activemask();
    const unsigned m = __ballot_sync(active, want);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(count, (unsigned long long)__popc(m));
    base = __shfl_sync(active, base, leader);
    if (want) {
        unsigned long long idx = base + __popc(m & ((1u << lane) - 1u));
        if ((int64_t)idx < cap) out[idx] = key;
    }
}

// Self pairs: thread p (sorted position) reports every leaf q > p whose
// exact box overlaps its own; subtrees whose sorted range ends at or before
// p are skipped, so each unordered pair is found once.
__global__ void k_self_pairs(const double* __restrict__ aabbs, Tree t, unsigned long long* count, uint64_t* out,
                             int64_t cap) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= t.n - 1) return;  // the last leaf has no later leaves
    const int op = t.sorted[p];
    double box[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) box[k] = aabbs[6 * (int64_t)op + k];
    const float4 qlo = t.leafbox[2 * p], qhi = t.leafbox[2 * p + 1];
    int stack[kStack];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const int node = stack[--sp];
        const int2 c = t.child[node];
        const int cc[2] = {c.x, c.y};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int x = cc[h];
            bool hit = false;
            uint64_t key = 0;
            if (x < 0) {
                const int64_t q = ~x;
                if (q > p) {
                    const int oq = t.sorted[q];
                    if (overlap64(box, aabbs + 6 * (int64_t)oq)) {
                        hit = true;
                        const uint32_t a = (uint32_t)min(op, oq), b = (uint32_t)max(op, oq);
                        key = ((uint64_t)a << 32) | b;
                    }
                }
            } else if (t.range[x].y > p && overlap32(qlo, qhi, t.box[2 * (int64_t)x], t.box[2 * (int64_t)x + 1])) {
                if (sp < kStack)
                    stack[sp++] = x;
                else
                    atomicExch(t.flags + 1, 1);
            }
            emit(hit, key, count, out, cap);
        }
    }
}

// Box queries: thread q reports every leaf whose exact box overlaps query q.
__global__ void k_query_boxes(const double* __restrict__ aabbs, Tree t, const double* __restrict__ boxes, int64_t m,
                              unsigned long long* count, uint64_t* out, int64_t cap) {
    int64_t qi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= m) return;
    double box[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) box[k] = boxes[6 * qi + k];
    const float4 qlo = make_float4(__double2float_rd(box[0]), __double2float_rd(box[2]), __double2float_rd(box[4]), 0.f);
    const float4 qhi = make_float4(__double2float_ru(box[1]), __double2float_ru(box[3]), __double2float_ru(box[5]), 0.f);
    if (t.n == 1) {
        const bool hit = overlap64(box, aabbs + 6 * (int64_t)t.sorted[0]);
        emit(hit, ((uint64_t)(uint32_t)t.sorted[0] << 32) | (uint32_t)qi, count, out, cap);
        return;
    }
    int stack[kStack];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const int node = stack[--sp];
        const int2 c = t.child[node];
        const int cc[2] = {c.x, c.y};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int x = cc[h];
            bool hit = false;
            uint64_t key = 0;
            if (x < 0) {
                const int ol = t.sorted[~x];
                if (overlap64(box, aabbs + 6 * (int64_t)ol)) {
                    hit = true;
                    key = ((uint64_t)(uint32_t)ol << 32) | (uint32_t)qi;
                }
            } else if (overlap32(qlo, qhi, t.box[2 * (int64_t)x], t.box[2 * (int64_t)x + 1])) {
                if (sp < kStack)
                    stack[sp++] = x;
                else
                    atomicExch(t.flags + 1, 1);
            }
            emit(hit, key, count, out, cap);
        }
    }
}

__global__ void k_decode(const uint64_t* __restrict__ keys, int64_t n, int32_t* __restrict__ pairs) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint64_t v = keys[k];
    pairs[2 * k] = (int32_t)(v >> 32);
    pairs[2 * k + 1] = (int32_t)(v & 0xffffffffu);
}

// Sort the hit keys and write int32 pairs; synchronises to read the count.
int finish_pairs(unsigned long long* d_count, uint64_t* keys, uint64_t* keys_alt, void* cub_temp, size_t cub_bytes,
                 int32_t* pairs, int64_t capacity, int64_t* n_pairs, const int32_t* flags, cudaStream_t st) {
    unsigned long long count = 0;
    int hflags[2] = {0, 0};
    cudaMemcpyAsync(&count, d_count, sizeof(count), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        d3d::set_error("bvh query: %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    if (n_pairs) *n_pairs = (int64_t)count;
    if (hflags[0] || hflags[1]) {
        d3d::set_error("bvh: traversal stack or refit bound exceeded (tree deeper than %d)", kStack);
        return D3D_ERR_CAPACITY;
    }
    if ((int64_t)count > capacity) {
        d3d::set_error("bvh query: %llu pairs exceed the capacity of %lld", count, (long long)capacity);
        return D3D_ERR_CAPACITY;
    }
    if (count == 0) return D3D_SUCCESS;
    size_t need = 0;
    cub::DeviceRadixSort::SortKeys(nullptr, need, keys, keys_alt, (int)count, 0, 64, st);
    if (need > cub_bytes) {
        d3d::set_error("bvh query: sort temporary storage too small");
        return D3D_ERR_CAPACITY;
    }
    e = cub::DeviceRadixSort::SortKeys(cub_temp, need, keys, keys_alt, (int)count, 0, 64, st);
    if (e != cudaSuccess) {
        d3d::set_error("bvh query: sort failed: %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    k_decode<<<d3d::grid_for((int64_t)count, kBlock), kBlock, 0, st>>>(keys_alt, (int64_t)count, pairs);
    return d3d::check_launch("bvh query");
}

size_t query_cub_bytes(int64_t capacity) {
    size_t b = 0;
    cub::DeviceRadixSort::SortKeys(nullptr, b, (const uint64_t*)nullptr, (uint64_t*)nullptr,
                                   (int)(capacity > 0 ? capacity : 1), 0, 64);
    return b;
}

}  // namespace

extern "C" size_t d3d_bvh_bytes(int64_t n_leaves) {
    if (n_leaves < 0 || n_leaves >= (int64_t(1) << 31)) return 0;
    return layout(nullptr, n_leaves, nullptr);
}

extern "C" int d3d_bvh_build(const double* aabbs, int64_t n, void* tree, size_t tree_bytes, void* stream) {
    D3D_REQUIRE(n >= 0 && n < (int64_t(1) << 31), "d3d_bvh_build: n out of range");
    D3D_REQUIRE(tree, "d3d_bvh_build: null tree buffer");
    size_t need = layout(nullptr, n, nullptr);
    if (tree_bytes < need) {
        d3d::set_error("d3d_bvh_build: tree buffer of %zu bytes < %zu", tree_bytes, need);
        return D3D_ERR_CAPACITY;
    }
    Tree t;
    layout(tree, n, &t);
    cudaStream_t st = d3d::as_stream(stream);
    cudaMemsetAsync(t.flags, 0, 4 * sizeof(int32_t), st);
    if (n == 0) return d3d::check_launch("d3d_bvh_build");
    D3D_REQUIRE(aabbs, "d3d_bvh_build: null aabbs");
    int blocks = (int)((n + kBlock - 1) / kBlock);
    if (blocks > kBoundBlocks) blocks = kBoundBlocks;
    k_center_bounds<<<blocks, kBlock, 0, st>>>(aabbs, n, t.bounds + 6);
    k_reduce_bounds<<<1, 32, 0, st>>>(t.bounds + 6, blocks, t.bounds);
    k_morton<<<d3d::grid_for(n, kBlock), kBlock, 0, st>>>(aabbs, n, t.bounds, t.keys, t.vals);
    size_t cub_bytes = t.cub_bytes;
    cudaError_t e = cub::DeviceRadixSort::SortPairs(t.cub_temp, cub_bytes, t.keys, t.keys_out, t.vals, t.sorted, (int)n,
                                                    0, 63, st);
    if (e != cudaSuccess) {
        d3d::set_error("d3d_bvh_build: sort failed: %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    k_leaf_boxes<<<d3d::grid_for(n, kBlock), kBlock, 0, st>>>(aabbs, n, t.sorted, t.leafbox);
    if (n > 1) {
        cudaMemsetAsync(t.parent, 0xff, sizeof(int32_t) * (size_t)(2 * n - 1), st);
        cudaMemsetAsync(t.visits, 0, sizeof(int32_t) * (size_t)(n - 1), st);
        k_karras<<<d3d::grid_for(n - 1, kBlock), kBlock, 0, st>>>(t.keys_out, n, t.child, t.range, t.parent);
        k_refit<<<d3d::grid_for(n, kBlock), kBlock, 0, st>>>(t);
    }
    return d3d::check_launch("d3d_bvh_build");
}

extern "C" int d3d_bvh_refit(const double* aabbs, int64_t n, void* tree, size_t tree_bytes, void* stream) {
    D3D_REQUIRE(n >= 0 && n < (int64_t(1) << 31), "d3d_bvh_refit: n out of range");
    D3D_REQUIRE(tree, "d3d_bvh_refit: null tree buffer");
    size_t need = layout(nullptr, n, nullptr);
    if (tree_bytes < need) {
        d3d::set_error("d3d_bvh_refit: tree buffer of %zu bytes < %zu", tree_bytes, need);
        return D3D_ERR_CAPACITY;
    }
    if (n == 0) return D3D_SUCCESS;
    D3D_REQUIRE(aabbs, "d3d_bvh_refit: null aabbs");
    Tree t;
    layout(tree, n, &t);
    cudaStream_t st = d3d::as_stream(stream);
    // same leaf order and topology; the boxes of leaves and nodes are redone
    k_leaf_boxes<<<d3d::grid_for(n, kBlock), kBlock, 0, st>>>(aabbs, n, t.sorted, t.leafbox);
    if (n > 1) {
        cudaMemsetAsync(t.visits, 0, sizeof(int32_t) * (size_t)(n - 1), st);
        k_refit<<<d3d::grid_for(n, kBlock), kBlock, 0, st>>>(t);
    }
    return d3d::check_launch("d3d_bvh_refit");
}

extern "C" size_t d3d_bvh_query_bytes(int64_t capacity) {
    if (capacity < 0) return 0;
    return 256 + 2 * up(sizeof(uint64_t) * (size_t)(capacity > 0 ? capacity : 1)) + up(query_cub_bytes(capacity));
}

static int query_common(const void* tree, int64_t n, int64_t capacity, void* scratch, size_t scratch_bytes,
                        Tree* t, unsigned long long** count, uint64_t** keys, uint64_t** alt, void** cub_temp,
                        size_t* cub_bytes) {
    D3D_REQUIRE(tree, "bvh query: null tree");
    D3D_REQUIRE(n >= 0 && capacity >= 0, "bvh query: negative size");
    size_t need = d3d_bvh_query_bytes(capacity);
    if (!scratch || scratch_bytes < need) {
        d3d::set_error("bvh query: scratch of %zu bytes < %zu", scratch_bytes, need);
        return D3D_ERR_CAPACITY;
    }
    layout(const_cast<void*>(tree), n, t);
    char* s = static_cast<char*>(scratch);
    *count = reinterpret_cast<unsigned long long*>(s);
    size_t kb = up(sizeof(uint64_t) * (size_t)(capacity > 0 ? capacity : 1));
    *keys = reinterpret_cast<uint64_t*>(s + 256);
    *alt = reinterpret_cast<uint64_t*>(s + 256 + kb);
    *cub_temp = s + 256 + 2 * kb;
    *cub_bytes = up(query_cub_bytes(capacity));
    return D3D_SUCCESS;
}

extern "C" int d3d_bvh_self_pairs(const double* aabbs, int64_t n, const void* tree, int32_t* pairs, int64_t capacity,
                                  int64_t* n_pairs, void* scratch, size_t scratch_bytes, void* stream) {
    Tree t;
    unsigned long long* count;
    uint64_t *keys, *alt;
    void* cub_temp;
    size_t cub_bytes;
    int rc = query_common(tree, n, capacity, scratch, scratch_bytes, &t, &count, &keys, &alt, &cub_temp, &cub_bytes);
    if (rc) return rc;
    cudaStream_t st = d3d::as_stream(stream);
    cudaMemsetAsync(count, 0, sizeof(unsigned long long), st);
    if (n > 1) {
        D3D_REQUIRE(aabbs && (pairs || capacity == 0), "d3d_bvh_self_pairs: null pointer");
        k_self_pairs<<<d3d::grid_for(n - 1, 128), 128, 0, st>>>(aabbs, t, count, keys, capacity);
        rc = d3d::check_launch("d3d_bvh_self_pairs");
        if (rc) return rc;
    }
    return finish_pairs(count, keys, alt, cub_temp, cub_bytes, pairs, capacity, n_pairs, t.flags, st);
}

extern "C" int d3d_bvh_query(const double* aabbs, int64_t n, const void* tree, const double* boxes, int64_t m,
                             int32_t* pairs, int64_t capacity, int64_t* n_pairs, void* scratch, size_t scratch_bytes,
                             void* stream) {
    Tree t;
    unsigned long long* count;
    uint64_t *keys, *alt;
    void* cub_temp;
    size_t cub_bytes;
    int rc = query_common(tree, n, capacity, scratch, scratch_bytes, &t, &count, &keys, &alt, &cub_temp, &cub_bytes);
    if (rc) return rc;
    D3D_REQUIRE(m >= 0 && m < (int64_t(1) << 31), "d3d_bvh_query: m out of range");
    cudaStream_t st = d3d::as_stream(stream);
    cudaMemsetAsync(count, 0, sizeof(unsigned long long), st);
    if (n > 0 && m > 0) {
        D3D_REQUIRE(aabbs && boxes && (pairs || capacity == 0), "d3d_bvh_query: null pointer");
        k_query_boxes<<<d3d::grid_for(m, 128), 128, 0, st>>>(aabbs, t, boxes, m, count, keys, capacity);
        rc = d3d::check_launch("d3d_bvh_query");
        if (rc) return rc;
    }
    return finish_pairs(count, keys, alt, cub_temp, cub_bytes, pairs, capacity, n_pairs, t.flags, st);
}
