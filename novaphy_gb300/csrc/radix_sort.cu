// Onesweep LSD radix sort (see radix_sort.cuh).
#include "radix_sort.cuh"

namespace pbf {

namespace {

constexpr uint32_t kFlagAggregate = 1u << 30;
constexpr uint32_t kFlagInclusive = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;
// Upper bound on polls of one predecessor's status word (~1 s at L2 latency).
// A tile only ever waits on tiles that started before it, so in a healthy run
// the wait is microseconds; on give-up the kernel records an error and writes
// nothing out of range.
constexpr int kLookbackSpinLimit = 1 << 21;

__device__ __forceinline__ uint32_t lane_mask_lt() {
    uint32_t m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ uint32_t load_status(const uint32_t* p) {
    return *reinterpret_cast<const volatile uint32_t*>(p);
}

__device__ __forceinline__ void store_status(uint32_t* p, uint32_t v) { atomicExch(p, v); }

// Exclusive prefix sum of one value per thread over a 256-thread block.
__device__ __forceinline__ uint32_t block_exclusive_scan_256(uint32_t v, uint32_t* s_warp) {
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    __syncthreads();  // s_warp may still be read by a previous scan
    uint32_t inc = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc += t;
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < 8 ? s_warp[lane] : 0u;
#pragma unroll
        for (int d = 1; d < 8; d <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= d) w += t;
        }
        if (lane < 8) s_warp[lane] = w;  // inclusive warp totals
    }
    __syncthreads();
    const uint32_t warp_excl = warp > 0 ? s_warp[warp - 1] : 0u;
    return warp_excl + inc - v;
}

template <class K>
__global__ void __launch_bounds__(kSortThreads)
k_sort_histogram(const K* __restrict__ keys, int n, int passes, uint32_t* __restrict__ hist) {
    __shared__ uint32_t sh[kSortMaxPasses][256];
    for (int i = threadIdx.x; i < kSortMaxPasses * 256; i += blockDim.x) (&sh[0][0])[i] = 0u;
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const K k = keys[i];
        for (int p = 0; p < passes; ++p) atomicAdd(&sh[p][(uint32_t)(k >> (8 * p)) & 255u], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
        const uint32_t c = (&sh[0][0])[i];
        if (c) atomicAdd(&hist[i], c);
    }
}

// One digit pass.  vals_in == nullptr means "values are the input positions".
template <class K>
__global__ void __launch_bounds__(kSortThreads)
k_onesweep(const K* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
           K* __restrict__ keys_out, uint32_t* __restrict__ vals_out, int n, int shift,
           const uint32_t* __restrict__ hist, uint32_t* lookback, uint32_t* tile_ctr,
           uint32_t* err) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_warp_hist[kSortThreads / 32][256];
    __shared__ uint32_t s_tile_excl[256];
    __shared__ uint32_t s_digit_base[256];
    __shared__ uint32_t s_scan[8];
    __shared__ K s_keys[kSortTile];
    __shared__ uint32_t s_vals[kSortTile];

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;

    if (tid == 0) s_tile = atomicAdd(tile_ctr, 1u);
    for (int i = tid; i < (kSortThreads / 32) * 256; i += kSortThreads)
        (&s_warp_hist[0][0])[i] = 0u;
    __syncthreads();
    const uint32_t tile = s_tile;
    const long long base = (long long)tile * kSortTile;

    // Load: warp w owns keys [base + 256w, base + 256w + 256), item k of lane l
    // at offset 32k + l, so ranking item by item keeps input order.
    K key[kSortItems];
    uint32_t val[kSortItems], rank[kSortItems];
    bool valid[kSortItems];
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const long long idx = base + warp * (32 * kSortItems) + k * 32 + lane;
        valid[k] = idx < n;
        key[k] = valid[k] ? keys_in[idx] : K(0);
        val[k] = valid[k] ? (vals_in ? vals_in[idx] : (uint32_t)idx) : 0u;
    }

    const uint32_t lt = lane_mask_lt();
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const uint32_t vmask = __ballot_sync(0xffffffffu, valid[k]);
        if (valid[k]) {
            const uint32_t d = (uint32_t)(key[k] >> shift) & 255u;
            const uint32_t peers = __match_any_sync(vmask, d);
            const uint32_t before = s_warp_hist[warp][d];
            rank[k] = before + __popc(peers & lt);
            __syncwarp(vmask);
            if (lane == __ffs(peers) - 1) s_warp_hist[warp][d] = before + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();

    // Per digit: exclusive offsets of the warps inside the tile, tile count.
    uint32_t count = 0;
    {
        const int d = tid;  // 256 threads, one digit each
        for (int w = 0; w < kSortThreads / 32; ++w) {
            const uint32_t t = s_warp_hist[w][d];
            s_warp_hist[w][d] = count;
            count += t;
        }
    }
    const uint32_t tile_excl = block_exclusive_scan_256(count, s_scan);
    s_tile_excl[tid] = tile_excl;

    // Decoupled look-back across tiles for digit `tid`.
    {
        uint32_t* my = lookback + (size_t)tile * 256 + tid;
        if (tile == 0) {
            store_status(my, kFlagInclusive | count);
        } else {
            store_status(my, kFlagAggregate | count);
        }
        uint32_t excl = 0;
        for (long long j = (long long)tile - 1; j >= 0; --j) {
            const uint32_t* st = lookback + (size_t)j * 256 + tid;
            uint32_t s = load_status(st);
            int spins = 0;
            while ((s & ~kValueMask) == 0u && spins < kLookbackSpinLimit) {
                ++spins;
                s = load_status(st);
            }
            if ((s & ~kValueMask) == 0u) {
                atomicOr(err, 1u);
                break;
            }
            excl += s & kValueMask;
            if ((s & ~kValueMask) == kFlagInclusive) break;
        }
        if (tile > 0) store_status(my, kFlagInclusive | ((excl + count) & kValueMask));
        // Global digit base: digits below d across all keys + this digit in
        // the preceding tiles.
        s_digit_base[tid] = excl;
    }
    const uint32_t digit_excl = block_exclusive_scan_256(hist[tid], s_scan);
    s_digit_base[tid] += digit_excl;
    __syncthreads();

    // Scatter to shared memory in tile-local sorted order.
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        if (valid[k]) {
            const uint32_t d = (uint32_t)(key[k] >> shift) & 255u;
            const uint32_t lp = s_tile_excl[d] + s_warp_hist[warp][d] + rank[k];
            if (lp < (uint32_t)kSortTile) {
                s_keys[lp] = key[k];
                s_vals[lp] = val[k];
            }
        }
    }
    __syncthreads();

    const long long rem = (long long)n - base;
    const int tile_n = rem < kSortTile ? (int)rem : kSortTile;
    for (int lp = tid; lp < tile_n; lp += kSortThreads) {
        const K k = s_keys[lp];
        const uint32_t d = (uint32_t)(k >> shift) & 255u;
        const uint32_t g = s_digit_base[d] + ((uint32_t)lp - s_tile_excl[d]);
        if (g < (uint32_t)n) {
            keys_out[g] = k;
            vals_out[g] = s_vals[lp];
        }
    }
}

}  // namespace

void sort_scratch_bind(SortScratch& s, void* base, int capacity) {
    const int cap = capacity > 0 ? capacity : 1;
    s.capacity = cap;
    s.tiles = (cap + kSortTile - 1) / kSortTile;
    char* p = reinterpret_cast<char*>(base);
    s.keys_alt = reinterpret_cast<void*>(p);
    p += sort_scratch_round((size_t)cap * 8);
    s.vals_alt = reinterpret_cast<uint32_t*>(p);
    p += sort_scratch_round((size_t)cap * 4);
    s.zeroed = reinterpret_cast<uint32_t*>(p);
    s.hist = reinterpret_cast<uint32_t*>(p);
    p += (size_t)kSortMaxPasses * 256 * 4;
    s.tile_ctr = reinterpret_cast<uint32_t*>(p);
    p += 64;
    s.err = reinterpret_cast<uint32_t*>(p);
    p += 64;
    s.lookback = reinterpret_cast<uint32_t*>(p);
    p += (size_t)kSortMaxPasses * (size_t)s.tiles * 256 * 4;
    s.zeroed_bytes = (size_t)(p - reinterpret_cast<char*>(s.zeroed));
}

template <class K>
static cudaError_t sort_impl(const K* keys_in, K* keys_out, uint32_t* vals_out, int n,
                             int key_bits, SortScratch& s, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    if (n > s.capacity || n > (int)kValueMask) return cudaErrorInvalidValue;
    int passes = (key_bits + 7) / 8;
    if (passes < 1) passes = 1;
    if (passes > (int)(sizeof(K) * 8 / 8) || passes > kSortMaxPasses) return cudaErrorInvalidValue;
    const int tiles = (n + kSortTile - 1) / kSortTile;
    // Zero the histograms and tile counters, and the look-back words of the
    // tiles this sort uses; keep the error word (cleared by its owner).
    cudaError_t e = cudaMemsetAsync(s.hist, 0, (size_t)kSortMaxPasses * 256 * 4 + 64, stream);
    if (e != cudaSuccess) return e;
    for (int p = 0; p < passes; ++p) {
        e = cudaMemsetAsync(s.lookback + (size_t)p * s.tiles * 256, 0, (size_t)tiles * 256 * 4,
                            stream);
        if (e != cudaSuccess) return e;
    }
    int hist_blocks = (n + kSortThreads * 16 - 1) / (kSortThreads * 16);
    if (hist_blocks > 1024) hist_blocks = 1024;
    k_sort_histogram<K><<<hist_blocks, kSortThreads, 0, stream>>>(keys_in, n, passes, s.hist);
    // Ping-pong so that the last pass writes keys_out / vals_out.
    const K* kin = keys_in;
    const uint32_t* vin = nullptr;
    K* alt = reinterpret_cast<K*>(s.keys_alt);
    for (int p = 0; p < passes; ++p) {
        const bool to_out = ((passes - 1 - p) % 2) == 0;
        K* kout = to_out ? keys_out : alt;
        uint32_t* vout = to_out ? vals_out : s.vals_alt;
        k_onesweep<K><<<tiles, kSortThreads, 0, stream>>>(
            kin, vin, kout, vout, n, 8 * p, s.hist + p * 256,
            s.lookback + (size_t)p * s.tiles * 256, s.tile_ctr + p, s.err);
        kin = kout;
        vin = vout;
    }
    return cudaGetLastError();
}

cudaError_t radix_sort_pairs(const uint32_t* keys_in, uint32_t* keys_out, uint32_t* vals_out,
                             int n, int key_bits, SortScratch& s, cudaStream_t stream) {
    return sort_impl<uint32_t>(keys_in, keys_out, vals_out, n, key_bits, s, stream);
}

cudaError_t radix_sort_pairs64(const unsigned long long* keys_in, unsigned long long* keys_out,
                               uint32_t* vals_out, int n, int key_bits, SortScratch& s,
                               cudaStream_t stream) {
    return sort_impl<unsigned long long>(keys_in, keys_out, vals_out, n, key_bits, s, stream);
}

}  // namespace pbf
