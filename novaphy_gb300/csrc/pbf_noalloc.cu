// Allocation-free variant of the cell-key sort (pbf_sort_pairs_noalloc).
//
// Who needs this: callers that must not allocate device memory while they
// run.  A host framework that owns every byte of device memory through its
// own pool (and accounts it against a budget) cannot let a library call
// cudaMalloc behind its back; a latency-bound loop cannot afford cudaMalloc /
// cudaFree either, because they can synchronize the whole device and can fail
// under memory pressure in the middle of a frame.  Such callers hand in device
// buffers they already own and get the sort done with no allocation at all.
//
// How: the sort's scratch (ping-pong key/value buffers, digit histograms,
// look-back words, tile counters, error word) lives in one file-scope
// __device__ array of fixed size, so every GPU that loads this library keeps
// kNoAllocScratchBytes reserved until the process exits.  Host code cannot use
// the array's name as a device address; the first call on each device, with
// that device current, looks the address up with cudaGetSymbolAddress and
// caches it.
//
// The call blocks: it waits for the sort on the caller's stream and reads the
// sort's error word back.  A stream that is being captured is refused.
//
// All calls share the one array and it keeps whatever the last call left in
// it: this entry clears the words that must start at zero on every call, and
// two calls whose work overlaps on the GPU (different streams or threads at
// the same time) race on the array and must be serialized by the caller.
// The keys and the two outputs must not overlap (no in-place sort).
#include <cstdint>
#include <mutex>
#include <string>

#include "novaphy_pbf.h"
#include "radix_sort.cuh"

namespace {

// Largest key count the static scratch can sort.
constexpr int kNoAllocMaxKeys = 1 << 18;  // 262,144 keys
// Exactly the scratch the sort carves for that many keys (sort_scratch_bind).
constexpr size_t kNoAllocScratchBytes = pbf::sort_scratch_bytes(kNoAllocMaxKeys);
static_assert(kNoAllocScratchBytes < (size_t)8 << 20, "static sort scratch above 8 MB");

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {};

}  // namespace

namespace pbf {
void set_last_error(const std::string& msg);  // pbf_last_error() text (pbf_capi.cu)
}  // namespace pbf

namespace {
struct ErrorSink {
    ErrorSink& operator=(const std::string& m) {
        pbf::set_last_error(m);
        return *this;
    }
} g_noalloc_error;
}  // namespace

extern "C" int pbf_sort_pairs_noalloc(int device, int n, const unsigned* d_keys, int key_bits,
                                      unsigned* d_out_keys, unsigned* d_out_vals, void* stream) {
    if (n < 0 || (n > 0 && (!d_keys || !d_out_keys || !d_out_vals))) {
        g_noalloc_error = "pbf_sort_pairs_noalloc: bad arguments";
        return PBF_ERR_INVALID_ARG;
    }
    if (key_bits < 1 || key_bits > 32) {
        g_noalloc_error = "pbf_sort_pairs_noalloc: key_bits must be in [1, 32]";
        return PBF_ERR_INVALID_ARG;
    }
    if (n > kNoAllocMaxKeys) {
        g_noalloc_error = "pbf_sort_pairs_noalloc: n = " + std::to_string(n) +
                          " exceeds the fixed maximum of " + std::to_string(kNoAllocMaxKeys) +
                          " keys of the allocation-free sort";
        return PBF_ERR_CAPACITY;
    }
    if (device < 0 || device >= kMaxDevices) {
        g_noalloc_error = "pbf_sort_pairs_noalloc: device out of range";
        return PBF_ERR_INVALID_ARG;
    }
    if (n == 0) return PBF_OK;
    // The first digit pass writes the outputs while other tiles still read
    // the keys, so the keys may not share memory with either output.
    const auto overlaps = [n](const void* a, const void* b) {
        const uintptr_t pa = reinterpret_cast<uintptr_t>(a), pb = reinterpret_cast<uintptr_t>(b);
        const uintptr_t len = (uintptr_t)n * sizeof(unsigned);
        return pa < pb + len && pb < pa + len;
    };
    if (overlaps(d_keys, d_out_keys) || overlaps(d_keys, d_out_vals) ||
        overlaps(d_out_keys, d_out_vals)) {
        g_noalloc_error = "pbf_sort_pairs_noalloc: d_keys, d_out_keys and d_out_vals must not "
                          "overlap (no in-place sort)";
        return PBF_ERR_INVALID_ARG;
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    {
        // The call waits for the sort and copies its error word back, which a
        // stream under capture does not allow: refuse instead of breaking the
        // caller's capture.
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
            g_noalloc_error = "pbf_sort_pairs_noalloc: the stream is being captured; this call "
                              "blocks until the sort is done and cannot be captured";
            return PBF_ERR_INVALID_ARG;
        }
    }
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        g_noalloc_error = std::string("pbf_sort_pairs_noalloc: cudaSetDevice: ") +
                          cudaGetErrorString(e);
        return PBF_ERR_NO_DEVICE;
    }
    int rc = PBF_OK;
    void* base = nullptr;
    {
        // One-time set-up per device, with that device current.
        std::lock_guard<std::mutex> lk(g_setup_mu);
        if (!g_scratch_addr[device]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                g_noalloc_error = std::string("pbf_sort_pairs_noalloc: cudaGetSymbolAddress: ") +
                                  cudaGetErrorString(e);
                rc = PBF_ERR_CUDA;
            } else {
                g_scratch_addr[device] = p;
            }
        }
        base = g_scratch_addr[device];
    }
    if (rc == PBF_OK) {
        pbf::SortScratch s;
        pbf::sort_scratch_bind(s, base, kNoAllocMaxKeys);
        // The array keeps the previous call's contents: the error word must
        // start at zero (the sort itself zeroes its histograms, tile counters
        // and look-back words).
        e = cudaMemsetAsync(s.err, 0, sizeof(uint32_t), st);
        if (e == cudaSuccess)
            e = pbf::radix_sort_pairs(d_keys, d_out_keys, d_out_vals, n, key_bits, s, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        uint32_t err = 0;
        if (e == cudaSuccess) e = cudaMemcpy(&err, s.err, sizeof(err), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            g_noalloc_error = std::string("pbf_sort_pairs_noalloc: ") + cudaGetErrorString(e);
            rc = PBF_ERR_CUDA;
        } else if (err) {
            g_noalloc_error = "pbf_sort_pairs_noalloc: a bounded device-side wait gave up";
            rc = PBF_ERR_TIMEOUT;
        }
    }
    if (prev >= 0) cudaSetDevice(prev);
    return rc;
}
