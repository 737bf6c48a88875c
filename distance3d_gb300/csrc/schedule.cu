// schedule.cu -- pair scheduling (type-sorted order), the library's scratch
// pool and persistent-launch sizing.
#include <cub/cub.cuh>

#include <mutex>

#include "capi_util.h"
#include "d3d_device.cuh"
#include "scratch.h"

namespace {

using d3d::pair_ok;

constexpr int kMaxDevices = 64;
std::mutex g_mu;
cudaMemPool_t g_pool[kMaxDevices] = {};

inline size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

std::mutex g_tune_mu;
d3d_tuning g_tuning = {128, 0, 4, 4096};

// key = ((type1 * 10 + type2) << 4) | size class of the larger hull or mesh
// (at most 99 * 16 + 15 < 2^11); slots at and beyond the device-side count (if given)
// get the largest key
__global__ void k_pair_keys(d3d_store s, const int32_t* __restrict__ i1, const int32_t* __restrict__ i2, int64_t n,
                            const int64_t* __restrict__ n_dev, uint32_t* __restrict__ keys,
                            int32_t* __restrict__ vals) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    vals[k] = (int32_t)k;
    if (n_dev && k >= *n_dev) {
        keys[k] = 0x7ffu;
        return;
    }
    const int ia = i1[k], ib = i2[k];
    if (!pair_ok(s, ia, ib)) {  // the kernels report the pair; its place in the order does not matter
        keys[k] = 0;
        return;
    }
    int4 a = __ldg(reinterpret_cast<const int4*>(s.meta) + ia);
    int4 b = __ldg(reinterpret_cast<const int4*>(s.meta) + ib);
    int nv = max(a.x == D3D_HULL || a.x == D3D_MESH ? a.y : 0, b.x == D3D_HULL || b.x == D3D_MESH ? b.y : 0);
    int cls = nv > 0 ? min(32 - __clz(nv), 15) : 0;
    unsigned ta = (unsigned)min(max(a.x, 0), D3D_MESH), tb = (unsigned)min(max(b.x, 0), D3D_MESH);
    keys[k] = ((ta * 10u + tb) << 4) | (unsigned)cls;
}

}  // namespace

namespace d3d {

int scratch_alloc(void** p, size_t bytes, cudaStream_t stream) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        set_error("scratch: no current device (%s)", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    cudaMemPool_t pool;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_pool[dev]) {
            cudaMemPoolProps props = {};
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            e = cudaMemPoolCreate(&g_pool[dev], &props);
            if (e != cudaSuccess) {
                g_pool[dev] = nullptr;
                set_error("scratch: cudaMemPoolCreate: %s", cudaGetErrorString(e));
                return D3D_ERR_CUDA;
            }
            uint64_t keep = uint64_t(1) << 30;
            cudaMemPoolSetAttribute(g_pool[dev], cudaMemPoolAttrReleaseThreshold, &keep);
        }
        pool = g_pool[dev];
    }
    e = cudaMallocFromPoolAsync(p, bytes ? bytes : 1, pool, stream);
    if (e != cudaSuccess) {
        set_error("scratch: allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    return D3D_SUCCESS;
}

void scratch_free(void* p, cudaStream_t stream) {
    if (p) cudaFreeAsync(p, stream);
}

int persistent_blocks(const void* kernel, int block, int64_t work_items, int max_per_sm, int smem) {
    int dev = 0, sms = 1, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
    if (max_per_sm > 0 && per_sm > max_per_sm) per_sm = max_per_sm;
    int64_t want = (work_items + block - 1) / block;
    int64_t full = (int64_t)sms * (per_sm > 0 ? per_sm : 1);
    int64_t b = want < full ? want : full;
    return (int)(b > 0 ? b : 1);
}

d3d_tuning tuning() {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    return g_tuning;
}

size_t pair_order_temp_bytes(int64_t n) {
    size_t cub_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (const int32_t*)nullptr, (int32_t*)nullptr, (int)n, 0, 11);
    return 2 * align_up(sizeof(uint32_t) * (size_t)n) + align_up(sizeof(int32_t) * (size_t)n) + align_up(cub_bytes);
}

int pair_order(const d3d_store& s, const int32_t* i1, const int32_t* i2, int64_t n, int32_t* order, void* temp,
               size_t temp_bytes, cudaStream_t stream, const int64_t* n_dev) {
    if (n <= 0) return D3D_SUCCESS;
    if (temp_bytes < pair_order_temp_bytes(n)) {
        set_error("pair_order: temporary storage too small");
        return D3D_ERR_CAPACITY;
    }
    char* t = static_cast<char*>(temp);
    uint32_t* keys = reinterpret_cast<uint32_t*>(t);
    t += align_up(sizeof(uint32_t) * (size_t)n);
    uint32_t* keys_out = reinterpret_cast<uint32_t*>(t);
    t += align_up(sizeof(uint32_t) * (size_t)n);
    int32_t* vals = reinterpret_cast<int32_t*>(t);
    t += align_up(sizeof(int32_t) * (size_t)n);
    size_t cub_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, keys, keys_out, vals, order, (int)n, 0, 11, stream);
    k_pair_keys<<<grid_for(n, 256), 256, 0, stream>>>(s, i1, i2, n, n_dev, keys, vals);
    cudaError_t e = cub::DeviceRadixSort::SortPairs(t, cub_bytes, keys, keys_out, vals, order, (int)n, 0, 11, stream);
    if (e != cudaSuccess) {
        set_error("pair_order: sort failed: %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    return check_launch("pair_order");
}

}  // namespace d3d

extern "C" int d3d_get_tuning(d3d_tuning* out) {
    D3D_REQUIRE(out, "d3d_get_tuning: null argument");
    *out = d3d::tuning();
    return D3D_SUCCESS;
}

extern "C" int d3d_set_tuning(const d3d_tuning* t) {
    D3D_REQUIRE(t, "d3d_set_tuning: null argument");
    D3D_REQUIRE(t->gjk_block == 64 || t->gjk_block == 128 || t->gjk_block == 256,
                "d3d_set_tuning: gjk_block must be 64, 128 or 256");
    D3D_REQUIRE(t->epa_warps == 2 || t->epa_warps == 4 || t->epa_warps == 8,
                "d3d_set_tuning: epa_warps must be 2, 4 or 8");
    D3D_REQUIRE(t->gjk_warps_per_sm >= 0 && t->sort_min >= 0, "d3d_set_tuning: negative value");
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tuning = *t;
    return D3D_SUCCESS;
}
