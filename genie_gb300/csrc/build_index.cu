// build_index.cu -- the CSR inverted index built on the device.
//
// Same result as build_host_index (host_index.cc): for every dim, a stable
// counting sort of the column by value, so ids ascend inside each (dim,value)
// list -- the layout of inv_list::invert + inv_table::build
// (table/inv_list.cc:295-320, table/inv_table.cu:267-350), which the reference
// runs single-threaded on the host with a copy of every list.
//
// Steps (values uploaded once, row-major n x d):
//   k_transpose   column-major copy (32x32 tiles through shared memory)
//   k_minmax      per-dim min / max
//   (host)        key_base from the ranges (one list per value in [min,max])
//   per dim j, chunks of kChunk objects:
//   k_hist        per-chunk histogram of the column's values (shared memory)
//   k_colscan     per value: exclusive sum over chunks -> each chunk's start
//                 inside the value's list; per-value totals
//   k_keyoff      exclusive scan of the totals -> key_off of the dim's lists
//   k_scatter     per chunk, in rounds of 1024 objects: sort (value, thread)
//                 pairs of the round, so an object's rank among equal values
//                 follows its id; place ids
// A dim whose value range exceeds kMaxBins falls back to the host builder.
#include "capi_internal.h"

#include <algorithm>

namespace gg {
namespace {

constexpr int kChunk = 4096;          // objects per chunk (one CTA)
constexpr int kMaxBins = 16384;       // values per dim the device path supports
constexpr int kBuildThreads = 1024;

__global__ void k_transpose(const int32_t *__restrict__ in, int32_t *__restrict__ out, int64_t n, int32_t d) {
    __shared__ int32_t tile[32][33];
    const int64_t r0 = (int64_t)blockIdx.x * 32, c0 = (int64_t)blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int64_t r = r0 + y, c = c0 + threadIdx.x;
        if (r < n && c < d) tile[y][threadIdx.x] = in[r * d + c];
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int64_t c = c0 + y, r = r0 + threadIdx.x;
        if (r < n && c < d) out[c * n + r] = tile[threadIdx.x][y];
    }
}

__global__ void k_minmax(const int32_t *__restrict__ col, int64_t n, int32_t *mn, int32_t *mx) {
    const int32_t j = blockIdx.y;
    const int32_t *c = col + (int64_t)j * n;
    int32_t lo = INT32_MAX, hi = INT32_MIN;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = c[i];
        lo = min(lo, v);
        hi = max(hi, v);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&mn[j], lo);
        atomicMax(&mx[j], hi);
    }
}

// H[c * bins + v] = objects of chunk c with value min + v
__global__ void __launch_bounds__(kBuildThreads) k_hist(const int32_t *__restrict__ col, int64_t n, int32_t vmin,
                                                         int32_t bins, uint32_t *H) {
    extern __shared__ uint32_t h[];
    for (int v = threadIdx.x; v < bins; v += blockDim.x) h[v] = 0;
    __syncthreads();
    const int64_t i0 = (int64_t)blockIdx.x * kChunk;
    const int64_t i1 = min(n, i0 + kChunk);
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) atomicAdd(&h[col[i] - vmin], 1u);
    __syncthreads();
    for (int v = threadIdx.x; v < bins; v += blockDim.x) H[(int64_t)blockIdx.x * bins + v] = h[v];
}

// per value: H becomes the exclusive sum over chunks; tot[v] = the total
__global__ void k_colscan(uint32_t *H, int64_t chunks, int32_t bins, int64_t *tot) {
    const int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= bins) return;
    int64_t s = 0;
    for (int64_t c = 0; c < chunks; ++c) {
        const uint32_t x = H[c * bins + v];
        H[c * bins + v] = (uint32_t)s;
        s += x;
    }
    tot[v] = s;
}

// key_off[kb + v] = base + exclusive sum of tot[0..v); one CTA
__global__ void __launch_bounds__(kBuildThreads) k_keyoff(const int64_t *tot, int32_t bins, int64_t base,
                                                           int64_t *key_off) {
    __shared__ int64_t carry_s;
    __shared__ int64_t warp_sum[32];
    if (threadIdx.x == 0) carry_s = base;
    __syncthreads();
    for (int32_t b0 = 0; b0 < bins; b0 += blockDim.x) {
        const int32_t v = b0 + threadIdx.x;
        const int64_t x = v < bins ? tot[v] : 0;
        int64_t incl = x;
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if ((threadIdx.x & 31) >= (unsigned)o) incl += y;
        }
        if ((threadIdx.x & 31) == 31) warp_sum[threadIdx.x >> 5] = incl;
        __syncthreads();
        if (threadIdx.x < 32) {
            const int nw = blockDim.x >> 5;
            int64_t w = threadIdx.x < (unsigned)nw ? warp_sum[threadIdx.x] : 0;
            int64_t wi = w;
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t y = __shfl_up_sync(0xffffffffu, wi, o);
                if (threadIdx.x >= (unsigned)o) wi += y;
            }
            if (threadIdx.x < (unsigned)nw) warp_sum[threadIdx.x] = wi - w;
        }
        __syncthreads();
        const int64_t before = carry_s + warp_sum[threadIdx.x >> 5] + incl - x;
        if (v < bins) key_off[v] = before;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry_s = before + x;
        __syncthreads();
    }
}

// Stable placement of chunk blockIdx.x's objects into the dim's lists.
__global__ void __launch_bounds__(kBuildThreads) k_scatter(const int32_t *__restrict__ col, int64_t n, int32_t vmin,
                                                            int32_t bins, const uint32_t *__restrict__ H,
                                                            const int64_t *__restrict__ key_off, uint32_t *ids) {
    extern __shared__ uint32_t run[];              // [bins] placed so far in this chunk, per value
    __shared__ uint32_t srt[kBuildThreads];        // (value << 10 | thread) of the round, sorted
    const uint32_t t = threadIdx.x;
    for (int v = t; v < bins; v += blockDim.x) run[v] = 0;
    const int64_t c = blockIdx.x;
    const int64_t i0 = c * kChunk, i1 = min(n, i0 + kChunk);
    for (int64_t r0 = i0; r0 < i1; r0 += kBuildThreads) {
        const int64_t i = r0 + t;
        const bool on = i < i1;
        const uint32_t v = on ? (uint32_t)(col[i] - vmin) : 0xFFFFFu;     // absent: after every value
        srt[t] = (v << 10) | t;
        // ascending bitonic sort of the round's 1024 keys
        for (uint32_t size = 2; size <= kBuildThreads; size <<= 1) {
            for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
                __syncthreads();
                const uint32_t p = t ^ stride;
                if (p > t) {
                    const uint32_t a = srt[t], b = srt[p];
                    const bool up = (t & size) == 0;
                    if ((a > b) == up) {
                        srt[t] = b;
                        srt[p] = a;
                    }
                }
            }
        }
        __syncthreads();
        // this thread's position in the sorted round, and where its value starts
        uint32_t lo = 0, hi = kBuildThreads;          // first key >= (v << 10)
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (srt[mid] < (v << 10)) lo = mid + 1; else hi = mid;
        }
        uint32_t me = lo, hi2 = kBuildThreads;        // this thread's own key
        const uint32_t key = (v << 10) | t;
        while (me < hi2) {
            const uint32_t mid = (me + hi2) >> 1;
            if (srt[mid] < key) me = mid + 1; else hi2 = mid;
        }
        if (on) {
            const uint32_t rank = me - lo;
            const int64_t pos = key_off[v] + H[c * bins + v] + run[v] + rank;
            ids[pos] = (uint32_t)i;
        }
        __syncthreads();
        // the first thread of each value in the round advances its counter
        if (on) {
            uint32_t e = lo, hi3 = kBuildThreads;     // first key > (v << 10 | 1023)
            const uint32_t last = (v << 10) | 1023u;
            while (e < hi3) {
                const uint32_t mid = (e + hi3) >> 1;
                if (srt[mid] <= last) e = mid + 1; else hi3 = mid;
            }
            if (me == lo) run[v] += e - lo;
        }
        __syncthreads();
    }
}

}  // namespace

// Device build of a one-value-per-object index; false when a dim's value
// range is beyond kMaxBins (the caller then builds on the host).  Fills the
// host mirror (bounds, key offsets) and the device arrays of ix.
int build_device_index(const int32_t *values, int64_t n, int32_t d, genie_index *ix, bool *used) {
    *used = false;
    cudaError_t e;
    static thread_local int prepared_device = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (prepared_device != dev) {     // per-value shared counters of up to kMaxBins values
        if ((e = cudaFuncSetAttribute((const void *)k_hist, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      kMaxBins * 4)) ||
            (e = cudaFuncSetAttribute((const void *)k_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      kMaxBins * 4)))
            return cuda_fail(e, "device index build");
        prepared_device = dev;
    }
    const size_t cells = (size_t)n * d;
    int32_t *d_vals = nullptr, *d_col = nullptr, *d_mn = nullptr, *d_mx = nullptr;
    auto cleanup = [&] {
        cudaFree(d_vals);
        cudaFree(d_col);
        cudaFree(d_mn);
        cudaFree(d_mx);
    };
    if ((e = cudaMalloc(&d_vals, cells * 4)) || (e = cudaMalloc(&d_col, cells * 4)) ||
        (e = cudaMalloc(&d_mn, d * 4)) || (e = cudaMalloc(&d_mx, d * 4))) {
        cleanup();
        return e == cudaErrorMemoryAllocation ? fail(GENIE_ERR_GPU_ALLOC, "device index build: out of memory")
                                              : cuda_fail(e, "device index build");
    }
    std::vector<int32_t> init_mn((size_t)d, INT32_MAX), init_mx((size_t)d, INT32_MIN);
    cudaMemcpy(d_vals, values, cells * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d_mn, init_mn.data(), d * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d_mx, init_mx.data(), d * 4, cudaMemcpyHostToDevice);
    k_transpose<<<dim3((unsigned)((n + 31) / 32), (unsigned)((d + 31) / 32)), dim3(32, 8)>>>(d_vals, d_col, n, d);
    cudaFree(d_vals);
    d_vals = nullptr;
    k_minmax<<<dim3((unsigned)std::min<int64_t>(1024, (n + 255) / 256), (unsigned)d), 256>>>(d_col, n, d_mn, d_mx);
    HostIndex &h = ix->host;
    h = HostIndex();
    h.n_objects = n;
    h.n_dims = d;
    h.mult_max = 1;
    h.dim_min.resize((size_t)d);
    h.dim_max.resize((size_t)d);
    cudaMemcpy(h.dim_min.data(), d_mn, d * 4, cudaMemcpyDeviceToHost);
    if ((e = cudaMemcpy(h.dim_max.data(), d_mx, d * 4, cudaMemcpyDeviceToHost))) {
        cleanup();
        return cuda_fail(e, "device index build");
    }
    for (int32_t j = 0; j < d; ++j)
        if ((int64_t)h.dim_max[j] - h.dim_min[j] + 1 > kMaxBins) {
            cleanup();
            return GENIE_OK;     // not used: the host builds this index
        }
    h.key_base.assign((size_t)d + 1, 0);
    for (int32_t j = 0; j < d; ++j) h.key_base[j + 1] = h.key_base[j] + ((int64_t)h.dim_max[j] - h.dim_min[j] + 1);
    const int64_t nk = h.n_keys();
    const int64_t chunks = (n + kChunk - 1) / kChunk;
    uint32_t *d_H = nullptr;
    int64_t *d_tot = nullptr, *d_keyoff = nullptr;
    if ((e = cudaMalloc(&d_H, (size_t)chunks * kMaxBins * 4)) || (e = cudaMalloc(&d_tot, kMaxBins * 8)) ||
        (e = ix->d_ids.reserve(cells * 4 + kIdsPadBytes)) || (e = ix->d_key_off.reserve((size_t)(nk + 1) * 8))) {
        cudaFree(d_H);
        cudaFree(d_tot);
        cleanup();
        return e == cudaErrorMemoryAllocation ? fail(GENIE_ERR_GPU_ALLOC, "device index build: out of memory")
                                              : cuda_fail(e, "device index build");
    }
    cudaMemset(ix->d_ids.p, 0, cells * 4 + kIdsPadBytes);
    d_keyoff = (int64_t *)ix->d_key_off.p;
    uint32_t *d_ids = (uint32_t *)ix->d_ids.p;
    for (int32_t j = 0; j < d; ++j) {
        const int32_t bins = (int32_t)(h.key_base[j + 1] - h.key_base[j]);
        const int32_t *col = d_col + (int64_t)j * n;
        const size_t hist_smem = (size_t)bins * 4;
        k_hist<<<(unsigned)chunks, kBuildThreads, hist_smem>>>(col, n, h.dim_min[j], bins, d_H);
        k_colscan<<<(unsigned)((bins + 255) / 256), 256>>>(d_H, chunks, bins, d_tot);
        k_keyoff<<<1, kBuildThreads>>>(d_tot, bins, (int64_t)j * n, d_keyoff + h.key_base[j]);
        k_scatter<<<(unsigned)chunks, kBuildThreads, hist_smem>>>(col, n, h.dim_min[j], bins, d_H,
                                                                  d_keyoff + h.key_base[j], d_ids);
    }
    const int64_t last = (int64_t)cells;
    cudaMemcpy(d_keyoff + nk, &last, 8, cudaMemcpyHostToDevice);
    e = cudaDeviceSynchronize();
    cudaFree(d_H);
    cudaFree(d_tot);
    cleanup();
    if (e) return cuda_fail(e, "device index build");
    h.key_off.resize((size_t)nk + 1);
    if ((e = cudaMemcpy(h.key_off.data(), d_keyoff, (size_t)(nk + 1) * 8, cudaMemcpyDeviceToHost)))
        return cuda_fail(e, "device index build");
    *used = true;
    return GENIE_OK;
}

}  // namespace gg
