// Onesweep LSD radix sort of (uint32 key, uint32 index) pairs.
//
// One histogram kernel counts the 8-bit digits of every pass in a single read
// of the keys; each digit pass is then ONE kernel: a tile of 2048 keys is
// ranked in shared memory (warp multisplit with __match_any_sync, stable in
// input order), the tile's per-digit counts are chained to the preceding
// tiles by decoupled look-back, and the tile is written out through shared
// memory so that each digit run is stored contiguously.
//
// The sort is stable, so ties keep input order: sorting cell keys of
// particles 0..n-1 yields, inside each cell, ascending particle index, which
// is the order the reference's hash buckets hold (neighbor_search.cpp:14-22).
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace pbf {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;  // 2048 keys per tile
constexpr int kSortMaxPasses = 8;

// Device scratch of one sorter, sized for `capacity` keys.
struct SortScratch {
    void* keys_alt = nullptr;      // ping-pong buffers (room for 64-bit keys)
    uint32_t* vals_alt = nullptr;
    uint32_t* zeroed = nullptr;    // hist | tile counters | look-back | error word
    size_t zeroed_bytes = 0;
    uint32_t* hist = nullptr;      // [kSortMaxPasses][256]
    uint32_t* tile_ctr = nullptr;  // [kSortMaxPasses]
    uint32_t* lookback = nullptr;  // [kSortMaxPasses][tiles][256]
    uint32_t* err = nullptr;       // bit 0: look-back wait gave up
    int capacity = 0;
    int tiles = 0;
};

// Bytes of one device allocation that sort_scratch_bind() carves into a
// sorter's scratch for `capacity` keys; each part starts on a 256-byte
// boundary.  constexpr, so a static array can be sized with it.
constexpr size_t sort_scratch_round(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t sort_scratch_bytes(int capacity) {
    const size_t cap = capacity > 0 ? (size_t)capacity : 1;
    const size_t tiles = (cap + kSortTile - 1) / kSortTile;
    return sort_scratch_round(cap * 8)                      // alt keys (room for 64-bit)
           + sort_scratch_round(cap * 4)                    // alt values
           + (size_t)kSortMaxPasses * 256 * 4               // hist
           + 64                                             // tile counters
           + 64                                             // error word
           + (size_t)kSortMaxPasses * tiles * 256 * 4;      // look-back
}
// Carves the scratch out of one device allocation of sort_scratch_bytes().
void sort_scratch_bind(SortScratch& s, void* base, int capacity);

// Sorts keys_in[0..n) (each < 2^key_bits).  Values are the input positions.
// Results land in keys_out / vals_out.  keys_in is not modified and may not
// alias the outputs.  Returns a CUDA error code (cudaSuccess on success).
cudaError_t radix_sort_pairs(const uint32_t* keys_in, uint32_t* keys_out, uint32_t* vals_out,
                             int n, int key_bits, SortScratch& s, cudaStream_t stream);
// Same for 64-bit keys (up to 8 digit passes).
cudaError_t radix_sort_pairs64(const unsigned long long* keys_in, unsigned long long* keys_out,
                               uint32_t* vals_out, int n, int key_bits, SortScratch& s,
                               cudaStream_t stream);

}  // namespace pbf
