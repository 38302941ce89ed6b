// PBF step kernels.  This file is compiled twice:
//   pbf_exact.cu: PBF_FAST=0, built with -fmad=false and IEEE div/sqrt, so
//                 every expression below rounds exactly like the reference's
//                 float code (pbf_solver.cpp, sph_kernel.h) term by term;
//   pbf_fast.cu:  PBF_FAST=1, built with FMA contraction, approximate
//                 division and square root, and rsqrt in the spiky gradient.
// Summation order is the reference's in both builds: for particle i the
// candidates are visited bucket by bucket over the 27 neighbour cells in
// (dz, dy, dx) order and, inside a bucket, by ascending particle index
// (neighbor_search.cpp:14-22, :36-48).
#pragma once

#include <cstdint>
#include <type_traits>

#include "exact_repeat.h"
#include "pbf_types.cuh"
#include "radix_sort.cuh"

#ifndef PBF_FAST
#error "define PBF_FAST before including pbf_kernels.cuh"
#endif
#ifndef PBF_NS
#error "define PBF_NS before including pbf_kernels.cuh"
#endif

namespace pbf {
namespace PBF_NS {

constexpr int kBlock = 128;
// A single scene of at least this many particles runs its neighbour passes
// with the warp-cooperative walk (and its one-thread fallback with the row
// loop unrolled by 8).  Smaller scenes and batches keep one thread per
// particle and the 4-way loop: many small scenes stepped side by side on their
// own streams run several kernels per SM at once, and there the larger code
// and shared memory measured up to 40 % slower.
constexpr int kBigScene = 1 << 17;
// The fewest candidates a row of the cooperative walk must hold before the
// walk looks for runs of identical candidates in it (rows of ordinary fluid
// hold a few hundred).
constexpr uint32_t kRunRow = 1024;
constexpr uint32_t kNoBucket = 0xffffffffu;
constexpr uint32_t kImpureBit = 0x80000000u;
// Flags in a particle's owner word (StepBuffers::sown) for runs of identical
// particles (k_segments): the particle only copies the results of its run's
// first particle (kCopyBit), or it is a run's first particle (kLeadBit).  The
// owner row itself takes the low 30 bits.
constexpr uint32_t kCopyBit = 0x40000000u;
constexpr uint32_t kLeadBit = 0x80000000u;
constexpr uint32_t kOwnerMask = 0x3fffffffu;
// Set in a slot's alias byte (StepBuffers::slot_alias, bit 0: alias) when the
// slot holds a run's first particle.
constexpr unsigned char kRunSlot = 2;

// ---------------------------------------------------------------------------
// SPH kernels (include/novaphy/fluid/sph_kernel.h:24-46)

// e0 + (e1 + e2): the 3-term reduction order of Vector3f::squaredNorm.
__device__ __forceinline__ float sqn(float x, float y, float z) { return x * x + (y * y + z * z); }

// r = x_i - x_j of a candidate and sqn(r), with (r.x, r.y) as one paired
// operation: fma(x_j, -1, x_i) rounds once, exactly as x_i - x_j, so the
// result is the reference's subtraction bit for bit.  The exact build also
// squares (r.x, r.y) as a pair; the _rn forms are never contracted, so the
// sum keeps sqn's separately rounded terms.  With with_w, rw = x_i.w + x_j.w
// (the lambda sum) comes from the same paired operation as r.z.
template <bool with_w = false>
__device__ __forceinline__ float rel_sq(const float4& xi, const float4& xj, float& rx, float& ry,
                                        float& rz, float* rw = nullptr) {
    const float2 dxy = __ffma2_rn(make_float2(xj.x, xj.y), make_float2(-1.0f, -1.0f),
                                  make_float2(xi.x, xi.y));
    rx = dxy.x;
    ry = dxy.y;
    if constexpr (with_w) {
        const float2 dzw = __ffma2_rn(make_float2(xj.z, xj.w), make_float2(-1.0f, 1.0f),
                                      make_float2(xi.z, xi.w));
        rz = dzw.x;
        *rw = dzw.y;
    } else {
        rz = xi.z - xj.z;
    }
#if PBF_FAST
    return sqn(rx, ry, rz);
#else
    const float2 sq = __fmul2_rn(dxy, dxy);
    return sq.x + (sq.y + rz * rz);
#endif
}

__device__ __forceinline__ float poly6(float r_sq, const StepConsts& C) {
    if (r_sq >= C.h2) return 0.0f;
    const float diff = C.h2 - r_sq;
    return C.k_poly * diff * diff * diff;
}

// Spiky gradient of r (= x_i - x_j) given r_sq = sqn(r); returns the scalar
// coefficient c so that grad = c * r (0 outside 1e-7 < |r| < h).
__device__ __forceinline__ float spiky_coeff(float r_sq, const StepConsts& C) {
#if PBF_FAST
    if (r_sq >= C.h2 || r_sq <= 1e-14f) return 0.0f;
    const float ir = rsqrtf(r_sq);
    const float diff = C.h - r_sq * ir;
    return C.k_spiky * diff * diff * ir;
#else
    const float r_len = sqrtf(r_sq);
    if (r_len <= 1e-7f || r_len >= C.h) return 0.0f;
    const float diff = C.h - r_len;
    return C.k_spiky * diff * diff / r_len;
#endif
}

// Adding a term to a running sum once (One) or m times in a row (a run of
// identical candidates in the cooperative walk): acc(s, t, m) is the float
// that m single additions of t leave, bit for bit.  (rep_add is inlined: as
// a call, the calling convention's saved registers cost the walk's hot
// loops spills.)
struct One {};
__device__ __forceinline__ float acc(float s, float t, One) { return s + t; }
__device__ __forceinline__ float acc(float s, float t, uint32_t m) { return rep_add(s, t, m); }
// The same as a call (the constraint passes' one-thread walks, where the
// inlined loop cost the density pass's hot loops registers).
struct Many {
    uint32_t n;
};
__device__ __noinline__ float rep_add_call(float s, float t, uint32_t m) { return rep_add(s, t, m); }
__device__ __forceinline__ float acc(float s, float t, Many m) { return rep_add_call(s, t, m.n); }

__device__ __forceinline__ bool bits_equal(const float4 a, const float4 b) {
    return __float_as_uint(a.x) == __float_as_uint(b.x) && __float_as_uint(a.y) == __float_as_uint(b.y) &&
           __float_as_uint(a.z) == __float_as_uint(b.z) && __float_as_uint(a.w) == __float_as_uint(b.w);
}

// ---------------------------------------------------------------------------
// Grid helpers

__device__ __forceinline__ int wrap(int c, int o, int g) {
    int t = (c - o) % g;
    return t < 0 ? t + g : t;
}

// Global slot of a cell: the grid's base plus its wrapped local index.
__device__ __forceinline__ uint32_t slot_of(int cx, int cy, int cz, const GridDesc& G) {
    return G.base + (uint32_t)wrap(cx, G.ox, G.gx) +
           (uint32_t)G.gx * ((uint32_t)wrap(cy, G.oy, G.gy) + (uint32_t)G.gy * (uint32_t)wrap(cz, G.oz, G.gz));
}

__device__ __forceinline__ bool in_grid(int cx, int cy, int cz, const GridDesc& G) {
    return (unsigned)(cx - G.ox) < (unsigned)G.gx && (unsigned)(cy - G.oy) < (unsigned)G.gy &&
           (unsigned)(cz - G.oz) < (unsigned)G.gz;
}

__device__ __forceinline__ void cell_of(float x, float y, float z, float inv, int& cx, int& cy,
                                        int& cz) {
    cx = (int)floorf(x * inv);
    cy = (int)floorf(y * inv);
    cz = (int)floorf(z * inv);
}

// Reference cell hash (neighbor_search.cpp:89-97).
__device__ __forceinline__ unsigned long long ref_hash(int cx, int cy, int cz) {
    return ((unsigned long long)(long long)cx * 73856093ULL) ^
           ((unsigned long long)(long long)cy * 19349663ULL) ^
           ((unsigned long long)(long long)cz * 83492791ULL);
}

// lower_bound over the sorted reference keys in [a, b).
__device__ __forceinline__ uint32_t key_lower_bound(const unsigned long long* __restrict__ keys,
                                                    uint32_t a, uint32_t b, unsigned long long k) {
    while (a < b) {
        const uint32_t m = (a + b) >> 1;
        if (__ldg(keys + m) < k) a = m + 1;
        else b = m;
    }
    return a;
}

// Visits the candidate sorted positions q of a particle whose step-start cell
// is `cell`, in the reference's order.  The particle itself is among them:
// the reference skips j == i in every pass but the density, and the kernels
// rely on its terms being exact zeros instead (spiky_grad(0) = 0 and the
// velocity / |omega| differences vanish), which leaves every sum unchanged.
//
// cell.w == 0 (clean): every neighbour bucket holds exactly the particles of
// that cell, so each (dz, dy) row of three cells is one contiguous range of
// the cell-sorted order.  cell.w == o + 1 (dirty: a neighbour key is shared
// with another occupied cell, or a slot holds wrapped aliases): the 27 bucket
// starts are row o of `btab`; a bucket is the run [start, bend) of the
// key-sorted order and kpos maps it back to cell-sorted positions.  U is the
// unroll factor of a row's candidate loop (see kBigScene).
template <int U = 4, class F>
__device__ __forceinline__ void for_each_candidate(const int4 cell, const uint32_t* __restrict__ off,
                                                   const uint32_t* __restrict__ kpos,
                                                   const uint32_t* __restrict__ bend,
                                                   const uint32_t* __restrict__ btab,
                                                   const StepConsts& C, F&& f) {
    const GridDesc& G = C.grid;
    if (cell.w == 0) {
        for (int dz = -1; dz <= 1; ++dz) {
            const uint32_t wz = (uint32_t)wrap(cell.z + dz, G.oz, G.gz);
            for (int dy = -1; dy <= 1; ++dy) {
                const uint32_t wy = (uint32_t)wrap(cell.y + dy, G.oy, G.gy);
                const uint32_t row = G.base + (uint32_t)G.gx * (wy + (uint32_t)G.gy * wz);
                const int wx = wrap(cell.x - 1, G.ox, G.gx);
                if (wx + 2 < G.gx) {
                    const uint32_t q1 = __ldg(off + row + wx + 3);
#pragma unroll U
                    for (uint32_t q = __ldg(off + row + wx); q < q1; ++q) f(q);
                } else {
                    for (int d = 0; d < 3; ++d) {
                        const uint32_t s = row + (uint32_t)wrap(cell.x - 1 + d, G.ox, G.gx);
                        const uint32_t q1 = __ldg(off + s + 1);
                        for (uint32_t q = __ldg(off + s); q < q1; ++q) f(q);
                    }
                }
            }
        }
    } else {
        const uint32_t* row = btab + (size_t)(uint32_t)(cell.w - 1) * 27u;
        for (int k = 0; k < 27; ++k) {
            const uint32_t b0 = __ldg(row + k);
            if (b0 == kNoBucket) continue;
            const uint32_t b1 = __ldg(bend + b0) & ~kImpureBit;
            for (uint32_t kq = b0; kq < b1; ++kq) f(__ldg(kpos + kq));
        }
    }
}

// ---------------------------------------------------------------------------
// Where a kernel finds its step constants and particle state.  One scene: the
// constants and the state arrays travel by value in the kernel parameters.
// A batch of scenes: tables with one entry per scene, indexed by the scene of
// the particle (sid, in the order the kernel walks); batch particle i of a
// scene whose particles start at `first` is the scene's particle i - first.

struct OneScene {
    StepConsts C;
    StateRef S;
    __device__ __forceinline__ const StepConsts& at(const uint32_t*, uint32_t) const { return C; }
    __device__ __forceinline__ const StateRef& state(const uint32_t*, uint32_t) const { return S; }
};

struct SceneTable {
    const StepConsts* __restrict__ tab;
    const StateRef* __restrict__ refs;
    __device__ __forceinline__ StepConsts at(const uint32_t* __restrict__ sid, uint32_t i) const {
        return tab[__ldg(sid + i)];
    }
    __device__ __forceinline__ StateRef state(const uint32_t* __restrict__ sid, uint32_t i) const {
        return refs[__ldg(sid + i)];
    }
};

// Scene ids of a step: per particle in particle order (pid) and in the
// cell-sorted order (spid); null for a single scene.
struct SceneIds {
    const uint32_t* __restrict__ pid;
    uint32_t* __restrict__ spid;
};

// ---------------------------------------------------------------------------
// Grid construction kernels

// v' = v + g dt;  x* = x + v' dt  (pbf_solver.cpp:31-32), rounded product
// then sum in both builds so that cell assignment is bit-exact.
__device__ __forceinline__ void predict(const float4 xi, const float4 vi, const StepConsts& C,
                                        float& px, float& py, float& pz) {
    const float vx = __fadd_rn(vi.x, __fmul_rn(C.g[0], C.dt));
    const float vy = __fadd_rn(vi.y, __fmul_rn(C.g[1], C.dt));
    const float vz = __fadd_rn(vi.z, __fmul_rn(C.g[2], C.dt));
    px = __fadd_rn(xi.x, __fmul_rn(vx, C.dt));
    py = __fadd_rn(xi.y, __fmul_rn(vy, C.dt));
    pz = __fadd_rn(xi.z, __fmul_rn(vz, C.dt));
}

// Predict + cell slot and reference hash key per particle (particle order).
template <class P>
__global__ void __launch_bounds__(kBlock)
k_predict_key(uint32_t* __restrict__ keys, unsigned long long* __restrict__ rkeys, int n,
              const SceneIds S, const P prm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const StepConsts& C = prm.at(S.pid, i);
    const StateRef& R = prm.state(S.pid, i);
    const uint32_t l = (uint32_t)i - R.first;
    float px, py, pz;
    predict(R.x[l], R.v[l], C, px, py, pz);
    int cx, cy, cz;
    cell_of(px, py, pz, C.inv_cell, cx, cy, cz);
    keys[i] = slot_of(cx, cy, cz, C.grid);
    rkeys[i] = ref_hash(cx, cy, cz);
}

// off[s] = lower_bound(skeys, s) for s in [0, nslots].
__global__ void __launch_bounds__(256)
k_offsets(const uint32_t* __restrict__ skeys, int n, uint32_t* __restrict__ off, uint32_t nslots) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > nslots) return;
    int a = 0, b = n;
    while (a < b) {
        const int m = (a + b) >> 1;
        if (__ldg(skeys + m) < s) a = m + 1;
        else b = m;
    }
    off[s] = (uint32_t)a;
}

// Gather particle state into cell-sorted order; recompute x* exactly as
// predicted.  Records each particle's sorted position (and scene) and flags
// slots that receive a particle from outside the grid box (wrapped alias).
template <class P>
__global__ void __launch_bounds__(kBlock)
k_gather(const uint32_t* __restrict__ sidx, float4* __restrict__ sx, float4* __restrict__ xa,
         float* __restrict__ srho, int4* __restrict__ scell, uint32_t* __restrict__ pos_of,
         unsigned char* __restrict__ slot_alias, uint32_t* __restrict__ err, int n,
         const SceneIds S, const P prm) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    uint32_t i = sidx[p];
    if (i >= (uint32_t)n) {  // only after a failed sort; keep every access in range
        atomicOr(err, 2u);
        i = 0;
    }
    const StepConsts& C = prm.at(S.pid, i);
    const StateRef& R = prm.state(S.pid, i);
    const uint32_t l = i - R.first;
    const float4 xi = R.x[l];
    float px, py, pz;
    predict(xi, R.v[l], C, px, py, pz);
    int cx, cy, cz;
    cell_of(px, py, pz, C.inv_cell, cx, cy, cz);
    sx[p] = make_float4(xi.x, xi.y, xi.z, __uint_as_float(i));
    xa[p] = make_float4(px, py, pz, R.lam[l]);
    srho[p] = R.rho[l];
    scell[p] = make_int4(cx, cy, cz, 0);
    pos_of[i] = (uint32_t)p;
    if (S.spid) S.spid[p] = S.pid[i];
    if (!in_grid(cx, cy, cz, C.grid)) slot_alias[slot_of(cx, cy, cz, C.grid)] = 1;
}

// Runs of particles with bit-identical step state (x, x* and lambda and rho
// as gathered) next to each other in cell order.  Everything a step computes
// for a particle follows from that state and from its candidates, which are
// those of its cell, so the particles of a run come out identical in every
// pass: only the run's first particle computes, and writes its results for
// the others too (their owner words get kCopyBit, the first one's segend the
// run's end).  Such runs form where the domain clamp piles fluid into a box
// corner, bit for bit: tens of thousands of particles, each of which would
// otherwise sum over all the others.  One warp per 32 positions; a warp with
// a run's first particle finds the run's end, 256 positions per round.
struct StepState {
    const float4* __restrict__ sx;
    const float4* __restrict__ xa;
    const float* __restrict__ srho;
    int n;
    __device__ __forceinline__ bool same(int a, int b) const {
        const float4 x0 = sx[a], x1 = sx[b], y0 = xa[a], y1 = xa[b];
        return __float_as_uint(x0.x) == __float_as_uint(x1.x) &&
               __float_as_uint(x0.y) == __float_as_uint(x1.y) &&
               __float_as_uint(x0.z) == __float_as_uint(x1.z) &&
               __float_as_uint(y0.x) == __float_as_uint(y1.x) &&
               __float_as_uint(y0.y) == __float_as_uint(y1.y) &&
               __float_as_uint(y0.z) == __float_as_uint(y1.z) &&
               __float_as_uint(y0.w) == __float_as_uint(y1.w) &&
               __float_as_uint(srho[a]) == __float_as_uint(srho[b]);
    }
};

__global__ void __launch_bounds__(256)
k_segments(const StepState S, const int4* __restrict__ scell, const GridDesc Gd,
           int* __restrict__ sown, unsigned char* __restrict__ slot_alias,
           uint32_t* __restrict__ segend) {
    const unsigned full = 0xffffffffu;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const bool in = p < S.n;
    const bool prev = in && p > 0 && S.same(p, p - 1);
    const bool next = in && p + 1 < S.n && S.same(p + 1, p);
    if (prev) sown[p] = (int)((uint32_t)sown[p] | kCopyBit);
    if (in && !prev && next) {
        sown[p] = (int)((uint32_t)sown[p] | kLeadBit);
        const int4 c = scell[p];
        unsigned char* a = slot_alias + slot_of(c.x, c.y, c.z, Gd);
        *a = (unsigned char)(*a | kRunSlot);
    }
    uint32_t end = 0u;
    uint32_t firsts = __ballot_sync(full, in && !prev && next);
    while (firsts) {
        const int l = __ffs(firsts) - 1;
        firsts &= firsts - 1u;
        // Positions from the first one's successor on, 8 per lane per round,
        // while each equals its predecessor.
        int base = (p - lane) + l + 1;
        int e = S.n;
        for (;;) {
            int fail = 8;
#pragma unroll
            for (int j = 7; j >= 0; --j) {
                const int q = base + lane * 8 + j;
                if (!(q < S.n && S.same(q, q - 1))) fail = j;
            }
            const uint32_t m = __ballot_sync(full, fail < 8);
            if (m) {
                const int fl = __ffs(m) - 1;
                e = base + fl * 8 + __shfl_sync(full, fail, fl);
                break;
            }
            base += 256;
        }
        if (lane == l) end = (uint32_t)e;
    }
    if (in) segend[p] = end;
}

// Reference buckets in key-sorted order: kpos maps key-sorted positions to
// cell-sorted ones; at each bucket start, bend holds the bucket end with
// kImpureBit set when the bucket mixes cells (hash collision).  With scene
// ids (ksid, in key-sorted order) a bucket never crosses a scene boundary:
// every scene has its own hash grid.  Two launches (enqueue_buckets): the
// bucket starts find their ends, then members whose cell differs from the
// previous member's mark their bucket impure.  Both searches gallop, so a
// bucket of L members costs O(log L) per thread; a serial scan by the start
// thread took milliseconds on buckets of tens of thousands of particles
// (fluid piled into a corner cell by the domain clamp).
struct BucketKeys {
    const unsigned long long* __restrict__ rsorted;
    const uint32_t* __restrict__ ksid;
    int n;
    __device__ __forceinline__ bool same(int m, unsigned long long k, uint32_t s0) const {
        return rsorted[m] == k && (!ksid || ksid[m] == s0);
    }
    // First position after kp outside kp's bucket.
    __device__ __forceinline__ int end_of(int kp) const {
        const unsigned long long k = rsorted[kp];
        const uint32_t s0 = ksid ? ksid[kp] : 0u;
        int lo = kp, step = 1, hi = kp + 1;
        while (hi < n && same(hi, k, s0)) {
            lo = hi;
            step <<= 1;
            hi = (n - kp > step) ? kp + step : n;
        }
        while (hi - lo > 1) {
            const int mid = lo + ((hi - lo) >> 1);
            if (same(mid, k, s0)) lo = mid;
            else hi = mid;
        }
        return hi;
    }
    // First position of kp's bucket.
    __device__ __forceinline__ int start_of(int kp) const {
        const unsigned long long k = rsorted[kp];
        const uint32_t s0 = ksid ? ksid[kp] : 0u;
        int hi = kp, step = 1, lo = kp - 1;
        while (lo >= 0 && same(lo, k, s0)) {
            hi = lo;
            step <<= 1;
            lo = (kp >= step) ? kp - step : -1;
        }
        while (hi - lo > 1) {
            const int mid = lo + ((hi - lo) >> 1);
            if (same(mid, k, s0)) hi = mid;
            else lo = mid;
        }
        return hi;
    }
};

__device__ __forceinline__ uint32_t cell_sorted_pos(const uint32_t* __restrict__ ridx,
                                                    const uint32_t* __restrict__ pos_of, int kp,
                                                    int n) {
    const uint32_t i0 = ridx[kp];
    uint32_t p0 = pos_of[i0 < (uint32_t)n ? i0 : 0];
    return p0 < (uint32_t)n ? p0 : 0u;
}

__global__ void __launch_bounds__(256)
k_buckets(const BucketKeys K, const uint32_t* __restrict__ ridx, const uint32_t* __restrict__ pos_of,
          uint32_t* __restrict__ kpos, uint32_t* __restrict__ bend) {
    const int kp = blockIdx.x * blockDim.x + threadIdx.x;
    if (kp >= K.n) return;
    kpos[kp] = cell_sorted_pos(ridx, pos_of, kp, K.n);
    if (kp > 0 && K.same(kp - 1, K.rsorted[kp], K.ksid ? K.ksid[kp] : 0u)) return;
    bend[kp] = (uint32_t)K.end_of(kp);
}

__global__ void __launch_bounds__(256)
k_bucket_mix(const BucketKeys K, const uint32_t* __restrict__ ridx,
             const uint32_t* __restrict__ pos_of, const int4* __restrict__ scell,
             uint32_t* __restrict__ bend) {
    const int kp = blockIdx.x * blockDim.x + threadIdx.x;
    if (kp == 0 || kp >= K.n) return;
    if (!K.same(kp - 1, K.rsorted[kp], K.ksid ? K.ksid[kp] : 0u)) return;
    const int4 c = scell[cell_sorted_pos(ridx, pos_of, kp, K.n)];
    const int4 d = scell[cell_sorted_pos(ridx, pos_of, kp - 1, K.n)];
    if (c.x != d.x || c.y != d.y || c.z != d.z) atomicOr(bend + K.start_of(kp), kImpureBit);
}

inline cudaError_t enqueue_buckets(const unsigned long long* rsorted, const uint32_t* ridx,
                                   const uint32_t* pos_of, const int4* scell,
                                   const uint32_t* ksid, uint32_t* kpos, uint32_t* bend, int n,
                                   cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const BucketKeys K{rsorted, ksid, n};
    const int nb = (n + 255) / 256;
    k_buckets<<<nb, 256, 0, st>>>(K, ridx, pos_of, kpos, bend);
    k_bucket_mix<<<nb, 256, 0, st>>>(K, ridx, pos_of, scell, bend);
    return cudaGetLastError();
}

// Marks query points whose neighbourhood differs from the reference's
// buckets over a source point set (qown[p] = owner + 1, else 0) and stores
// their 27 bucket starts in row `owner` of btab.  Query cells are qcell[0..nq),
// the source's key-sorted buckets are (rsorted, kpos, bend) with cells scell
// and slot alias flags of the source's grid; a query of scene s searches the
// scene's key range [seg_begin, seg_end).  Within a warp, one lane per
// distinct cell (and scene) does the 27 lookups; the other lanes reuse its row.
template <class P>
__global__ void __launch_bounds__(kBlock)
k_classify(const int4* __restrict__ qcell, int nq, const int4* __restrict__ scell,
           const unsigned long long* __restrict__ rsorted, const uint32_t* __restrict__ kpos,
           const uint32_t* __restrict__ bend, const unsigned char* __restrict__ slot_alias,
           uint32_t* __restrict__ btab, int* __restrict__ qown, const uint32_t* __restrict__ qsid,
           const P prm) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = p < (uint32_t)nq;
    const int lane = threadIdx.x & 31;
    const int4 cell = active ? qcell[p] : make_int4(0x7fffffff, 0x7fffffff, 0x7fffffff, 0);
    const uint32_t sc = (active && qsid) ? qsid[p] : 0xffffffffu;
    const unsigned long long kxy =
        ((unsigned long long)(unsigned)cell.x << 32) | (unsigned long long)(unsigned)cell.y;
    const unsigned full = 0xffffffffu;
    const uint32_t same = __match_any_sync(full, kxy) & __match_any_sync(full, (unsigned)cell.z) &
                          __match_any_sync(full, sc) & __ballot_sync(full, active);
    const int leader = same ? __ffs(same) - 1 : lane;
    // Each distinct cell of the warp in turn (its first lane is the owner of
    // its bucket row); lanes 0..26 look up one neighbour bucket each, m =
    // 9 (dz + 1) + 3 (dy + 1) + (dx + 1), so the 27 searches run side by side.
    uint32_t todo = __ballot_sync(full, active && lane == leader);
    int own = 0;
    while (todo) {
        const int L = __ffs(todo) - 1;
        todo &= todo - 1u;
        const uint32_t lp = __shfl_sync(full, p, L);
        const int cx = __shfl_sync(full, cell.x, L);
        const int cy = __shfl_sync(full, cell.y, L);
        const int cz = __shfl_sync(full, cell.z, L);
        const uint32_t grp = __shfl_sync(full, same, L);
        const StepConsts& C = prm.at(qsid, lp);
        int dirty = 0;
        if (C.hash_compat) {
            uint32_t t = kNoBucket;
            if (lane < 27) {
                const int nx = cx + lane % 3 - 1, ny = cy + (lane / 3) % 3 - 1, nz = cz + lane / 9 - 1;
                const unsigned long long k = ref_hash(nx, ny, nz);
                const uint32_t lb = key_lower_bound(rsorted, C.seg_begin, C.seg_end, k);
                if (lb < C.seg_end && __ldg(rsorted + lb) == k) {
                    t = lb;
                    const uint32_t e = __ldg(bend + lb);
                    const int4 c0 = scell[__ldg(kpos + lb)];
                    if ((e & kImpureBit) || c0.x != nx || c0.y != ny || c0.z != nz) dirty = 1;
                }
                if (slot_alias[slot_of(nx, ny, nz, C.grid)]) dirty = 1;
            }
            dirty = __any_sync(full, dirty);
            if (dirty && lane < 27) btab[(size_t)lp * 27u + (uint32_t)lane] = t;
        }
        if ((grp >> lane) & 1u) own = dirty ? (int)(lp + 1u) : 0;
    }
    if (active) qown[p] = own;
}

// ---------------------------------------------------------------------------
// Constraint and velocity kernels (one thread per cell-sorted particle)

struct Grid {
    const int4* __restrict__ scell;
    const int* __restrict__ sown;
    const uint32_t* __restrict__ off;
    const uint32_t* __restrict__ kpos;
    const uint32_t* __restrict__ bend;
    const uint32_t* __restrict__ btab;
    const uint32_t* __restrict__ spid;  // scene of each sorted particle (batches)
    uint32_t* moved;                     // per slot, see StepBuffers::moved
    uint32_t* lamnz;                     // per slot, see StepBuffers::lamnz
    BoundaryGrid bg;                     // two-way coupled steps only
    uint32_t* dhist;                     // see StepBuffers::dhist
    const uint32_t* segend;              // see StepBuffers::segend (large single scenes)
    const unsigned char* slot_alias;     // with kRunSlot where segend is set
};

// for_each_candidate over a single scene's step with runs of identical
// particles (k_segments): in a cell range or a one-cell bucket of at least
// kRunRow candidates, a run's first particle q calls fr(q, L) for the run's L
// particles, which come next in the candidate order (the run lies in one
// cell, in cell order), and the walk goes on after them.
template <int U, bool kRuns, class F, class FR>
__device__ __forceinline__ void for_each_candidate_runs(const int4 cell, const Grid& G,
                                                        const StepConsts& C, F&& f, FR&& fr) {
    if constexpr (!kRuns) {
        for_each_candidate<U>(cell, G.off, G.kpos, G.bend, G.btab, C, f);
        return;
    }
    if (!G.segend) {
        for_each_candidate<U>(cell, G.off, G.kpos, G.bend, G.btab, C, f);
        return;
    }
    const GridDesc& Gd = C.grid;
    // Slots [s, s + k) of a cell range [q, q1): only ranges with a run's
    // first particle read the run flags of their candidates.
    auto range = [&](uint32_t q, uint32_t q1, uint32_t s, int k) {
        bool any = false;
        if (q1 - q >= kRunRow)
            for (int d = 0; d < k; ++d) any |= (__ldg(G.slot_alias + s + d) & kRunSlot) != 0;
        if (!any) {
#pragma unroll U
            for (; q < q1; ++q) f(q);
            return;
        }
        while (q < q1) {
            if ((uint32_t)__ldg(G.sown + q) & kLeadBit) {
                const uint32_t e = __ldg(G.segend + q);
                fr(q, e - q);
                q = e;
            } else {
                f(q);
                ++q;
            }
        }
    };
    if (cell.w == 0) {
        for (int dz = -1; dz <= 1; ++dz) {
            const uint32_t wz = (uint32_t)wrap(cell.z + dz, Gd.oz, Gd.gz);
            for (int dy = -1; dy <= 1; ++dy) {
                const uint32_t wy = (uint32_t)wrap(cell.y + dy, Gd.oy, Gd.gy);
                const uint32_t row = Gd.base + (uint32_t)Gd.gx * (wy + (uint32_t)Gd.gy * wz);
                const int wx = wrap(cell.x - 1, Gd.ox, Gd.gx);
                if (wx + 2 < Gd.gx) {
                    range(__ldg(G.off + row + wx), __ldg(G.off + row + wx + 3), row + wx, 3);
                } else {
                    for (int d = 0; d < 3; ++d) {
                        const uint32_t s = row + (uint32_t)wrap(cell.x - 1 + d, Gd.ox, Gd.gx);
                        range(__ldg(G.off + s), __ldg(G.off + s + 1), s, 1);
                    }
                }
            }
        }
    } else {
        const uint32_t* row = G.btab + (size_t)(uint32_t)(cell.w - 1) * 27u;
        for (int k = 0; k < 27; ++k) {
            const uint32_t b0 = __ldg(row + k);
            if (b0 == kNoBucket) continue;
            const uint32_t be = __ldg(G.bend + b0);
            const uint32_t b1 = be & ~kImpureBit;
            bool any = false;
            if (!(be & kImpureBit) && b1 - b0 >= kRunRow) {
                const int4 c = G.scell[__ldg(G.kpos + b0)];
                any = (__ldg(G.slot_alias + slot_of(c.x, c.y, c.z, Gd)) & kRunSlot) != 0;
            }
            if (!any) {
                for (uint32_t kq = b0; kq < b1; ++kq) f(__ldg(G.kpos + kq));
                continue;
            }
            // One cell's members, in cell order: a run's particles follow its
            // first one here too.
            for (uint32_t kq = b0; kq < b1;) {
                const uint32_t q = __ldg(G.kpos + kq);
                if ((uint32_t)__ldg(G.sown + q) & kLeadBit) {
                    const uint32_t L = __ldg(G.segend + q) - q;
                    fr(q, L);
                    kq += L;
                } else {
                    f(q);
                    ++kq;
                }
            }
        }
    }
}

// The run flags of sorted particle p (kCopyBit, kLeadBit).
__device__ __forceinline__ uint32_t run_flags(const Grid& G, uint32_t p) {
    return (uint32_t)G.sown[p] & ~kOwnerMask;
}

// One past the last particle of the run p leads (p + 1 when it leads none).
__device__ __forceinline__ uint32_t run_end(const Grid& G, uint32_t p, uint32_t flags) {
    return (flags & kLeadBit) ? __ldg(G.segend + p) : p + 1;
}

// The cell of sorted particle p against the boundary index (two-way steps).
__device__ __forceinline__ int4 boundary_cell(const Grid& G, uint32_t p, const int4 cell) {
    const uint32_t i = __float_as_uint(__ldg(&G.bg.sx[p].w));
    return make_int4(cell.x, cell.y, cell.z, __ldg(G.bg.own + i));
}

__device__ __forceinline__ int4 cell_at(const Grid& G, uint32_t p) {
    int4 c = G.scell[p];
    c.w = (int)((uint32_t)G.sown[p] & kOwnerMask);
    return c;
}

// Load of a step array that the Jacobi loop rewrites.  Per-pass kernels read
// it through the read-only cache (nothing writes it during their launch); the
// persistent loop, whose other blocks rewrite it between its passes, uses
// plain loads, which its grid barrier orders after those writes.
template <bool kPersist, class T>
__device__ __forceinline__ T ld_step(const T* p) {
    if constexpr (kPersist) return *p;
    else return __ldg(p);
}

// ---------------------------------------------------------------------------
// Warp-cooperative candidate walk (single scenes).
//
// The 32 particles of a warp usually sit in one cell, or in two or three
// cells next to each other along x.  When every lane is clean (no merged
// reference bucket near it) and the lanes' cells share one (y, z) row and
// span at most three cells in x, the lanes' candidate sequences are
// sub-sequences of one sequence: the 9 rows (dz, dy) of cells
// [xmin - 1, xmax + 1], each in slot order, which is the reference's order
// (cells in (dz, dy, dx) order, ascending particle index inside a cell).  A
// lane's own sequence is that one restricted to the cells within one of its
// own in x.  The warp walks it in two phases:
//
//  1. listing, chunk by chunk: each lane loads one candidate per round of 32
//     (coalesced); a candidate farther from the bounding box of the warp's
//     positions than the kernel support adds an exact zero to every lane and
//     is dropped, the rest are staged in shared memory in order (x, y and z
//     in separate arrays), up to CH per chunk, and their positions appended
//     to the warp's survivor list.  Each lane then tests the chunk's
//     candidates two at a time (paired f32x2 operations) and sets a bit in
//     its own mask over the survivor list for each one that may be in its
//     support and lies in its own 27 cells.  The test is conservative: it
//     fuses the squares and sums (a few ulps from the exact r^2) and compares
//     against the support radius widened by 1e-6, so it keeps every
//     in-support candidate, and every term re-tests the exact r^2 itself;
//  2. evaluation, once the list holds up to CAP survivors or the walk ends:
//     each lane evaluates the terms of its set bits in order, loading each
//     candidate by its position one term ahead.
//
// Every lane thus adds exactly the nonzero terms of the one-thread walk, in
// the same order, so the sums are bit-identical.  The terms (two IEEE
// divisions and a square root in the exact build) run with the lanes of a
// step busy instead of waiting on the few in-support lanes of each
// candidate, and the distance test runs on the surviving candidates only.
// The list spans the whole walk rather than one chunk because the candidate
// order is spatially coherent: a chunk covers a few rows, which lie in the
// support of some lanes and not of others, so evaluating chunk by chunk
// leaves many lanes of each term step idle.  Only single scenes of at least
// kBigScene particles walk cooperatively (see CoopBlock).

// Candidates staged per chunk, and survivors listed before an evaluation:
// shared memory is CH * 17 + CAP * 8 bytes per warp (6.98 KB), eight blocks
// of four warps per SM (each block also takes 1 KB of the SM's 228 KB).  (128-candidate chunks pad less but fit seven
// blocks per SM, and measured slower.)
constexpr int coop_chunk(int) { return 64; }
constexpr int kCoopCap = 736;

template <int CH, bool kExtra>
struct CoopSmem {
    static constexpr int kCap = CH > 1 ? kCoopCap : 1;
    alignas(16) float sx[CH];          // staged x* of the chunk, by component; slots past
    alignas(16) float sy[CH];          // the last staged one up to a multiple of 32
    alignas(16) float sz[CH];          // hold +inf (never in support)
    alignas(16) float sw[CH];          // staged x*.w (lambda in the delta pass)
    unsigned char c[CH];               // cell of the candidate among [xmin - 1, xmax + 1]
    uint32_t q[kCap];                  // candidate position of each listed survivor
    uint32_t mask[(kCap + 31) / 32][32];  // mask[w][lane] bit b: survivor 32 w + b is a term of the lane
};

// Blocks per SM the neighbour-pass kernels are compiled for: 32 warps per SM
// (64 registers a thread), which their shared memory also fits.
template <int BS>
constexpr int kPassMinBlocks = 1024 / BS;

// Shared memory of a kernel's warps: real for the kernels of a single large
// scene (those with the 8-way row loop, see kBigScene), one byte otherwise.
// Small scenes and batches keep the one-thread walk: the shared memory costs
// them occupancy (a batch of 1,024 small scenes ran at 94 M particle-steps/s
// with the cooperative walk against 108 M without), and many small scenes
// side by side on their own streams measured slower with it too.
template <class P, int BS, bool kExtra, int U>
struct CoopBlock {
    static constexpr bool kOn = std::is_same<P, OneScene>::value && U == 8;
    using Smem = CoopSmem<kOn ? coop_chunk(BS) : 1, kExtra>;
    static constexpr int kWarps = kOn ? BS / 32 : 1;
};

// The warp's shared row: cells y = cy, z = cz, x in [xmin, xmin + W - 3];
// wx0 = wrapped x slot of xmin - 1.
struct CoopRow {
    int cy, cz, xmin, W, wx0;
};

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Warp-collective (every lane of the warp must call it): whether the warp
// walks cooperatively, and its row.  `cell` is the lane's step-start cell
// with w = its owner row (0 = clean); `sid` its scene (0 for a single scene):
// the lanes must share one scene, whose grid is Gd.
__device__ __forceinline__ bool coop_row(bool active, const int4 cell, const GridDesc& Gd,
                                         CoopRow& R, uint32_t sid) {
    const unsigned full = 0xffffffffu;
    if (!__all_sync(full, active)) return false;
    if (!__all_sync(full, sid == __shfl_sync(full, sid, 0))) return false;
    const int cy0 = __shfl_sync(full, cell.y, 0);
    const int cz0 = __shfl_sync(full, cell.z, 0);
    if (!__all_sync(full, cell.w == 0 && cell.y == cy0 && cell.z == cz0)) return false;
    const int xmin = __reduce_min_sync(full, cell.x);
    const int xmax = __reduce_max_sync(full, cell.x);
    if ((long long)xmax - (long long)xmin > 2 || xmin <= -(1 << 30) || xmax >= (1 << 30))
        return false;
    const int W = xmax - xmin + 3;
    const int wx0 = wrap(xmin - 1, Gd.ox, Gd.gx);
    if (wx0 + W > Gd.gx) return false;  // the row range would wrap: one-thread walk
    R = CoopRow{cy0, cz0, xmin, W, wx0};
    return true;
}

// The cooperative walk (see above) of a warp for which coop_row held.  xi is
// the lane's x*, ci its cell x; `cut` the support test r_sq < cut of the
// pass.  extra(q) returns the per-candidate extras of candidate q (kExtra);
// body(xj, ej) adds the term of one candidate, re-testing r_sq < cut;
// rep(xj, ej, L) adds it L times in a row (exactly, see acc).
// Lanes with `want` false list no candidates and do not widen the warp's
// box (at least one lane must want).
// kRuns: rows of at least kRunRow candidates collapse runs of identical
// candidates (below).  The XSPH and vorticity passes compile it in; the
// constraint passes do not (it cost their register allocation about 4 %
// of their time on ordinary fluid).
// kLam (the delta pass): a candidate whose lambda sum with the lane,
// xi.w + xj.w, is zero adds an exact zero to the lane's sum (no s_corr
// either, which needs a negative sum), and the sum, started at +0, never is
// -0, so such candidates are not listed; when every lane's lambda is zero,
// candidates with zero lambda are not staged at all.
template <int CH, bool kExtra, bool kPersist, bool kLam, bool kRuns, class Extra, class Body,
          class Rep>
__device__ __forceinline__ void coop_walk(CoopSmem<CH, kExtra>& sm, const CoopRow& R, int ci,
                                          const float4 xi, const float4* xin, float cut,
                                          const GridDesc& Gd, const uint32_t* __restrict__ off,
                                          Extra&& extra, Body&& body, Rep&& rep,
                                          bool want = true) {
    constexpr int CAP = CoopSmem<CH, kExtra>::kCap;
    static_assert(CH % 32 == 0 && CAP % 32 == 0 && CAP >= 2 * CH, "coop walk sizes");
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const float inf = __int_as_float(0x7f800000);
    float lx = want ? xi.x : inf, ly = want ? xi.y : inf, lz = want ? xi.z : inf;
    float hx = want ? xi.x : -inf, hy = want ? xi.y : -inf, hz = want ? xi.z : -inf;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        lx = fminf(lx, __shfl_xor_sync(full, lx, o));
        ly = fminf(ly, __shfl_xor_sync(full, ly, o));
        lz = fminf(lz, __shfl_xor_sync(full, lz, o));
        hx = fmaxf(hx, __shfl_xor_sync(full, hx, o));
        hy = fmaxf(hy, __shfl_xor_sync(full, hy, o));
        hz = fmaxf(hz, __shfl_xor_sync(full, hz, o));
    }
    // A candidate in some lane's support is within sqrt(cut) of the box, and
    // within the widened radius of the lane's fused r^2; the margins cover
    // the rounding of both distance computations.
    const float lim = cut * 1.001f;
    const float lim2 = cut * 1.000001f;
    const bool all_member = R.W == 3;  // one cell: every staged candidate is in it
    const int myc = ci - R.xmin + 1;   // the lane's cell among the row's cells
    const uint32_t lt = lanemask_lt();
    const float2 m1 = make_float2(-1.0f, -1.0f);
    const float2 px = make_float2(xi.x, xi.x), py = make_float2(xi.y, xi.y),
                 pz = make_float2(xi.z, xi.z), pw = make_float2(xi.w, xi.w);
    // Only candidates with a nonzero lambda can add to a lane whose own is zero.
    const bool lam_filter = kLam && !__any_sync(full, xi.w != 0.0f);
    int nst = 0;   // staged in the current chunk
    int base = 0;  // survivors listed so far (a multiple of 32)
    int cnt = 0;   // the lane's listed terms

    // Phase 2: every lane evaluates its listed terms in list order, loading
    // the next term's candidate before adding the current one.
    auto evaluate = [&]() {
        const int most = (int)__reduce_max_sync(full, (unsigned)cnt);
        int w = 0;
        uint32_t bits = sm.mask[0][lane];
        auto next_q = [&]() {
            while (bits == 0) bits = sm.mask[++w][lane];
            const int k = 32 * w + __ffs(bits) - 1;
            bits &= bits - 1u;
            return sm.q[k];
        };
        float4 xn = make_float4(0.0f, 0.0f, 0.0f, 0.0f), en = xn;
        if (cnt > 0) {
            const uint32_t q = next_q();
            xn = ld_step<kPersist>(xin + q);
            if constexpr (kExtra) en = extra(q);
        }
        for (int t = 0; t < most; ++t) {
            const float4 xj = xn, ej = en;
            if (t + 1 < cnt) {
                const uint32_t q = next_q();
                xn = ld_step<kPersist>(xin + q);
                if constexpr (kExtra) en = extra(q);
            }
            if (t < cnt) body(xj, ej);
        }
        __syncwarp();
        cnt = 0;
        base = 0;
    };

    // Phase 1b: the lane's support tests over the staged chunk, two
    // candidates per paired operation, one mask word per 32 candidates.  Only
    // whole words are tested until the walk ends: the last partial word's
    // candidates move to the front of the stage (their list positions stay
    // where they are, at base + k) and wait for the next chunk, so a tested
    // word is padded only at the very end of the walk.
    auto test_chunk = [&](bool last) {
        const int words = last ? (nst + 31) >> 5 : nst >> 5;
        if (last) {
            // Pad the last word with candidates that are never in support.
            for (int k = nst + lane; k < (words << 5); k += 32) {
                sm.sx[k] = __int_as_float(0x7f800000);
                sm.sy[k] = 0.0f;
                sm.sz[k] = 0.0f;
                sm.sw[k] = 0.0f;
                sm.c[k] = 0;
            }
            __syncwarp();
        }
        for (int wd = 0; wd < words; ++wd) {
            const int k0 = wd << 5;
            uint32_t allowed = full;
            if (!all_member) {
                // Candidates of the word in each of the row's cells (at most
                // 5), then those in the lane's three.
                const int cc = sm.c[k0 + lane];
                allowed = 0u;
#pragma unroll
                for (int v = 0; v < 5; ++v) {
                    const uint32_t mc = __ballot_sync(full, cc == v);
                    if ((unsigned)(v - myc + 1) <= 2u) allowed |= mc;
                }
            }
            uint32_t bits = 0u;
#pragma unroll
            for (int b = 0; b < 32; b += 2) {
                const float2 X = *reinterpret_cast<const float2*>(&sm.sx[k0 + b]);
                const float2 Y = *reinterpret_cast<const float2*>(&sm.sy[k0 + b]);
                const float2 Z = *reinterpret_cast<const float2*>(&sm.sz[k0 + b]);
                const float2 dx = __ffma2_rn(X, m1, px);
                const float2 dy = __ffma2_rn(Y, m1, py);
                const float2 dz = __ffma2_rn(Z, m1, pz);
                float2 r2 = __fmul2_rn(dx, dx);
                r2 = __ffma2_rn(dy, dy, r2);
                r2 = __ffma2_rn(dz, dz, r2);
                if constexpr (kLam) {
                    const float2 W = *reinterpret_cast<const float2*>(&sm.sw[k0 + b]);
                    const float2 ls = __fadd2_rn(pw, W);
                    if (r2.x < lim2 && ls.x != 0.0f) bits |= 1u << b;
                    if (r2.y < lim2 && ls.y != 0.0f) bits |= 2u << b;
                } else {
                    if (r2.x < lim2) bits |= 1u << b;
                    if (r2.y < lim2) bits |= 2u << b;
                }
            }
            bits &= allowed;
            if (!want) bits = 0u;
            sm.mask[(base >> 5) + wd][lane] = bits;
            cnt += __popc(bits);
        }
        // The untested rest (fewer than 32) moves to the front of the stage.
        const int rest = last ? 0 : nst - (words << 5);
        float kx = 0.0f, ky = 0.0f, kz = 0.0f, kw = 0.0f;
        unsigned char kc = 0;
        uint32_t kq = 0u;
        if (lane < rest) {
            const int k = (words << 5) + lane;
            kx = sm.sx[k];
            ky = sm.sy[k];
            kz = sm.sz[k];
            kw = sm.sw[k];
            kc = sm.c[k];
            kq = sm.q[base + k];
        }
        __syncwarp();
        base += words << 5;
        if (base > CAP - CH) evaluate();
        if (lane < rest) {
            sm.sx[lane] = kx;
            sm.sy[lane] = ky;
            sm.sz[lane] = kz;
            sm.sw[lane] = kw;
            sm.c[lane] = kc;
            sm.q[base + lane] = kq;
        }
        nst = rest;
        __syncwarp();
    };

    for (int rr = 0; rr < 9; ++rr) {
        const int dz = rr / 3 - 1;
        const int dy = rr - (rr / 3) * 3 - 1;
        const uint32_t row = Gd.base + (uint32_t)R.wx0 +
                             (uint32_t)Gd.gx * ((uint32_t)wrap(R.cy + dy, Gd.oy, Gd.gy) +
                                                (uint32_t)Gd.gy * (uint32_t)wrap(R.cz + dz, Gd.oz, Gd.gz));
        const uint32_t q0 = __ldg(off + row);
        const uint32_t q1 = __ldg(off + row + R.W);
        // Cell boundaries inside the row (cells 1.. W-1 start here).
        uint32_t b1 = q1, b2 = q1, b3 = q1, b4 = q1;
        if (!all_member) {
            b1 = __ldg(off + row + 1);
            b2 = __ldg(off + row + 2);
            b3 = __ldg(off + row + 3);
            if (R.W > 4) b4 = __ldg(off + row + 4);
        }
        // Stages the candidates q of the lanes with `ok` that pass the box.
        auto stage = [&](uint32_t q, bool ok) {
            bool pass = false;
            float4 xj = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (ok) {
                xj = ld_step<kPersist>(xin + q);
                const float ex = fmaxf(0.0f, fmaxf(lx - xj.x, xj.x - hx));
                const float ey = fmaxf(0.0f, fmaxf(ly - xj.y, xj.y - hy));
                const float ez = fmaxf(0.0f, fmaxf(lz - xj.z, xj.z - hz));
                pass = ex * ex + (ey * ey + ez * ez) < lim;
                if (lam_filter) pass = pass && xj.w != 0.0f;
            }
            const uint32_t m = __ballot_sync(full, pass);
            if (pass) {
                const int k = nst + __popc(m & lt);
                sm.sx[k] = xj.x;
                sm.sy[k] = xj.y;
                sm.sz[k] = xj.z;
                sm.sw[k] = xj.w;
                sm.q[base + k] = q;
                sm.c[k] = (unsigned char)((q >= b1) + (q >= b2) + (q >= b3) + (q >= b4));
            }
            nst += __popc(m);
            if (nst >= 32) {
                __syncwarp();
                test_chunk(false);
            }
        };
        if (!kRuns || q1 - q0 < kRunRow) {
            for (uint32_t qb = q0; qb < q1; qb += 32) stage(qb + (uint32_t)lane, qb + lane < q1);
        } else {
            // (kRuns) A row long enough to hold a run of identical
            // candidates: the domain clamp piles fluid into a box corner, bit
            // for bit, and such a cell holds tens of thousands.  Candidates with the same
            // (xj, ej) in the same cell add the same term to a lane, so a
            // run of whole 32-candidate chunks of them is not staged: the
            // candidates before it are settled first, then each lane adds
            // the run's term as many times as the run is long (rep, an exact
            // repeated addition), then the walk goes on.  Shorter runs and
            // run ends inside a chunk are staged as usual.
            bool inrun = false;
            float4 rx = make_float4(0.0f, 0.0f, 0.0f, 0.0f), re = rx;
            uint32_t rn = 0;
            int rc = 0;
            auto apply = [&]() {
                if (want && (all_member || (unsigned)(rc - myc + 1) <= 2u)) rep(rx, re, rn);
                __syncwarp();
                inrun = false;
            };
            for (uint32_t qb = q0; qb < q1; qb += 32) {
                const uint32_t q = qb + (uint32_t)lane;
                const bool ok = q < q1;
                float4 xj = make_float4(0.0f, 0.0f, 0.0f, 0.0f), ej = xj;
                if (ok) {
                    xj = ld_step<kPersist>(xin + q);
                    if constexpr (kExtra) ej = extra(q);
                }
                const int cq = (int)((q >= b1) + (q >= b2) + (q >= b3) + (q >= b4));
                float4 ax = rx, ae = re;
                int ac = rc;
                if (!inrun) {
                    ax = make_float4(__shfl_sync(full, xj.x, 0), __shfl_sync(full, xj.y, 0),
                                     __shfl_sync(full, xj.z, 0), __shfl_sync(full, xj.w, 0));
                    if constexpr (kExtra)
                        ae = make_float4(__shfl_sync(full, ej.x, 0), __shfl_sync(full, ej.y, 0),
                                         __shfl_sync(full, ej.z, 0), __shfl_sync(full, ej.w, 0));
                    ac = __shfl_sync(full, cq, 0);
                }
                const bool same = ok && cq == ac && bits_equal(xj, ax) && (!kExtra || bits_equal(ej, ae));
                const uint32_t sm_same = __ballot_sync(full, same);
                if (inrun) {
                    if (sm_same == full) {
                        rn += 32;
                        continue;
                    }
                    const int f = __ffs(~sm_same) - 1;  // the run ends before lane f
                    rn += (uint32_t)f;
                    apply();
                    stage(q, ok && lane >= f);
                } else if (sm_same == full) {
                    if (nst > 0) {
                        __syncwarp();
                        test_chunk(true);
                    }
                    if (base > 0) evaluate();
                    inrun = true;
                    rx = ax;
                    re = ae;
                    rc = ac;
                    rn = 32;
                } else {
                    stage(q, ok);
                }
            }
            if (inrun) apply();
        }
    }
    if (nst > 0) {
        __syncwarp();
        test_chunk(true);
    }
    if (base > 0) evaluate();
}

// Scene of sorted particle p (0 for a single scene).
__device__ __forceinline__ uint32_t scene_at(const Grid& G, uint32_t p) {
    return G.spid ? __ldg(G.spid + p) : 0u;
}

// Whether a slot among the 27 around a clean particle's cell holds the stamp
// `it`: with the moved stamps and it, whether a candidate moved in the delta
// pass of Jacobi iteration it - 1 (when none did, the candidates all sit
// where they sat for the previous density pass, so the particle's rho and
// lambda would come out bit for bit the same); with the lambda stamps and
// it + 1, whether a candidate has a nonzero lambda in iteration it.
template <bool kPersist>
__device__ __forceinline__ bool neighbourhood_moved(const int4 cell, const GridDesc& Gd,
                                                    const uint32_t* moved, int it) {
    // The 27 slots from 3 wrapped coordinates per axis; the loads are
    // independent, so they overlap.
    uint32_t wx[3], wy[3], wz[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        wx[d] = (uint32_t)wrap(cell.x + d - 1, Gd.ox, Gd.gx);
        wy[d] = (uint32_t)wrap(cell.y + d - 1, Gd.oy, Gd.gy);
        wz[d] = (uint32_t)wrap(cell.z + d - 1, Gd.oz, Gd.gz);
    }
    bool any = false;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const uint32_t row = Gd.base + (uint32_t)Gd.gx * (wy[b] + (uint32_t)Gd.gy * wz[c]);
#pragma unroll
            for (int a = 0; a < 3; ++a)
                any |= ld_step<kPersist>(moved + row + wx[a]) == (uint32_t)it;
        }
    return any;
}

// compute_density + compute_lambda (pbf_solver.cpp:129-179) in one candidate
// pass for sorted particle p.  Reads x* from xin, writes (x*, lambda) to xout
// and rho to srho.  Scenes whose `iters` are done by iteration `it` are left
// untouched.  Warp-collective: every lane of the warp calls it, with
// `active` false past the last particle.
template <bool kPersist, int U, class P, int CH>
__device__ __forceinline__ void density_lambda_at(uint32_t p, bool active, const float4* xin,
                                                  float4* xout, float* __restrict__ srho, int it,
                                                  const Grid& G, const P& prm,
                                                  CoopSmem<CH, false>& sm) {
    constexpr bool kCoop = CoopBlock<P, 32, false, U>::kOn;
    const uint32_t pa = active ? p : 0u;
    const StepConsts& C = prm.at(G.spid, pa);
    const int4 cell = cell_at(G, pa);
    const uint32_t rf = run_flags(G, pa);
    bool live = active && it < C.iters && !(rf & kCopyBit);
    if (live && it > 0 && G.moved && cell.w == 0 &&
        !neighbourhood_moved<kPersist>(cell, C.grid, G.moved, it)) {
        // Nothing around moved since the last density pass: keep its rho
        // (srho) and lambda (x*.w, which the delta pass carried through).
        const float4 keep = xin[p];
        xout[p] = keep;
        for (uint32_t m = p + 1, e = run_end(G, p, rf); m < e; ++m) xout[m] = keep;
        if (G.lamnz && keep.w != 0.0f)
            G.lamnz[slot_of(cell.x, cell.y, cell.z, C.grid)] = (uint32_t)it + 1u;
        live = false;
    }
    CoopRow R;
    bool coop = false;
    if constexpr (kCoop) coop = coop_row(live, cell, C.grid, R, scene_at(G, pa));
    if (!live) return;
    const float4 xi = xin[p];
    float density = 0.0f, sum_grad_sq = 0.0f, gix = 0.0f, giy = 0.0f, giz = 0.0f;
    float ci_first = 0.0f;  // C_i of a density-first walk (computed once)
    bool have_ci = false;
    // The term of candidate xj, added L times (One: once); density-first
    // walks add the density alone (grads false) or the gradient sums alone.
    auto part = [&](const float4& xj, auto L, bool dens, bool grads) {
        float rx, ry, rz;
        const float r_sq = rel_sq(xi, xj, rx, ry, rz);
        if (r_sq < C.cut) {
            if (dens) density = acc(density, C.mass * poly6(r_sq, C), L);
            if (grads) {
                const float c = spiky_coeff(r_sq, C);
                const float gx = C.mr * (c * rx);
                const float gy = C.mr * (c * ry);
                const float gz = C.mr * (c * rz);
                sum_grad_sq = acc(sum_grad_sq, sqn(gx, gy, gz), L);
                gix = acc(gix, gx, L);
                giy = acc(giy, gy, L);
                giz = acc(giz, gz, L);
            }
        }
    };
    auto term = [&](const float4& xj, auto L) { part(xj, L, true, true); };
    if constexpr (kCoop) {
        if (coop) {
            auto none = [](uint32_t) { return float4{}; };
            // Density first: when C_i < 0 lambda_i is 0 whatever the gradient
            // sums, so a warp can sum the densities alone (poly6 terms, no
            // square root or division), then walk again, in the same
            // candidate order, for the gradients of its lanes with
            // C_i >= 0 only.  Each sum sees the same terms in the same order
            // as the single walk: same bits.  It pays where most warps have
            // no such lane; which way a warp goes follows the share of
            // warps that needed gradients in the same iteration of the last
            // step.
            bool dfirst = false;
            if (G.dhist && it < kWalkHist && !G.bg.spos) {
                const uint32_t need = __ldg(G.dhist + it), ran = __ldg(G.dhist + kWalkHist + it);
                dfirst = ran > 0 && 3u * need < ran;
            }
            auto once = [&](const float4& xj, const float4&) { term(xj, One{}); };
            // (The walk is compiled without runs here, kRuns false, so `times`
            // is never called; it states what a run would add.)
            auto times = [&](const float4& xj, const float4&, uint32_t L) { term(xj, L); };
            if (!dfirst) {
                coop_walk<CH, false, kPersist, false, false>(sm, R, cell.x, xi, xin, C.cut, C.grid, G.off,
                                                      none, once, times);
            } else {
                // Densities only, then gradients only for the lanes that want.
                bool want = true, grads = false;
                for (;;) {
                    coop_walk<CH, false, kPersist, false, false>(
                        sm, R, cell.x, xi, xin, C.cut, C.grid, G.off, none,
                        [&](const float4& xj, const float4&) {
                            float rx, ry, rz;
                            const float r_sq = rel_sq(xi, xj, rx, ry, rz);
                            if (r_sq < C.cut) {
                                if (!grads) {
                                    density += C.mass * poly6(r_sq, C);
                                } else {
                                    const float c = spiky_coeff(r_sq, C);
                                    const float gx = C.mr * (c * rx);
                                    const float gy = C.mr * (c * ry);
                                    const float gz = C.mr * (c * rz);
                                    sum_grad_sq += sqn(gx, gy, gz);
                                    gix += gx;
                                    giy += gy;
                                    giz += gz;
                                }
                            }
                        },
                        [&](const float4& xj, const float4&, uint32_t L) {
                            part(xj, L, !grads, grads);
                        },
                        want);
                    if (grads) break;
                    ci_first = density * C.inv_rho0 - 1.0f;
                    have_ci = true;
                    want = !(ci_first < 0.0f);
                    if (!__any_sync(0xffffffffu, want)) break;
                    grads = true;
                }
            }
            if (G.dhist && it < kWalkHist && (threadIdx.x & 31) == 0) {
                atomicAdd(G.dhist + 3 * kWalkHist + it, 1u);
            }
        }
    }
    if (!coop)
        for_each_candidate_runs<U, std::is_same<P, OneScene>::value>(
            cell, G, C, [&](uint32_t q) { term(ld_step<kPersist>(xin + q), One{}); },
            [&](uint32_t q, uint32_t L) { term(ld_step<kPersist>(xin + q), Many{L}); });
    if (G.bg.spos) {
        // Two-way coupling (no counterpart in the reference): after the fluid
        // terms, the boundary's Akinci density rho0 psi_b W and its gradient
        // psi_b grad W (= (rho0 psi_b / rho0) grad W) in the boundary index's
        // bucket order.  The boundary does not move, so it adds nothing to
        // the sum of the neighbours' squared gradients.
        for_each_candidate<4>(boundary_cell(G, p, cell), G.bg.off, G.bg.kpos, G.bg.bend,
                              G.bg.btab, C, [&](uint32_t q) {
                                  const float4 b = __ldg(G.bg.spos + q);
                                  const float rx = xi.x - b.x, ry = xi.y - b.y, rz = xi.z - b.z;
                                  const float r_sq = sqn(rx, ry, rz);
                                  if (r_sq < C.cut) {
                                      density += C.rho0 * b.w * poly6(r_sq, C);
                                      const float c = spiky_coeff(r_sq, C);
                                      gix += b.w * (c * rx);
                                      giy += b.w * (c * ry);
                                      giz += b.w * (c * rz);
                                  }
                              });
    }
    sum_grad_sq += sqn(gix, giy, giz);
    const float Ci = have_ci ? ci_first : density * C.inv_rho0 - 1.0f;
    const float lam = (Ci < 0.0f) ? 0.0f : -Ci / (sum_grad_sq + C.eps);
    if constexpr (kCoop) {
        if (coop && G.dhist && it < kWalkHist &&
            __any_sync(0xffffffffu, !(Ci < 0.0f)) && (threadIdx.x & 31) == 0)
            atomicAdd(G.dhist + 2 * kWalkHist + it, 1u);
    }
    if (G.lamnz && lam != 0.0f) G.lamnz[slot_of(cell.x, cell.y, cell.z, C.grid)] = (uint32_t)it + 1u;
    srho[p] = density;
    xout[p] = make_float4(xi.x, xi.y, xi.z, lam);
    for (uint32_t m = p + 1, e = run_end(G, p, rf); m < e; ++m) {
        srho[m] = density;
        xout[m] = make_float4(xi.x, xi.y, xi.z, lam);
    }
}

template <int BS, class P, int U = 4>
__global__ void __launch_bounds__(BS, kPassMinBlocks<BS>)
k_density_lambda(const float4* __restrict__ xin, float4* __restrict__ xout, float* __restrict__ srho,
                 int it, int n, const Grid G, const P prm) {
    using B = CoopBlock<P, BS, false, U>;
    __shared__ typename B::Smem sm[B::kWarps];
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    density_lambda_at<false, U>(p, p < (uint32_t)n, xin, xout, srho, it, G, prm,
                                sm[B::kOn ? threadIdx.x >> 5 : 0]);
}

// Velocity update with speed clamp (pbf_solver.cpp:81-93) for sorted p; w is
// the XSPH weight m / rho' (pbf_solver.cpp:240-241).
__device__ __forceinline__ float4 update_velocity(float px, float py, float pz, const float4 x0,
                                                  float rho, const StepConsts& C) {
    float a = (px - x0.x) * C.inv_dt;
    float b = (py - x0.y) * C.inv_dt;
    float c = (pz - x0.z) * C.inv_dt;
    const float speed_sq = sqn(a, b, c);
    if (speed_sq > C.max_speed_sq) {
        const float s = C.max_speed / sqrtf(speed_sq);
        a *= s;
        b *= s;
        c *= s;
    }
    const float rho_j = (rho > 1e-6f) ? rho : C.rho0;
    return make_float4(a, b, c, C.mass / rho_j);
}

// compute_delta_position + apply_delta (pbf_solver.cpp:181-223, :74-76) for
// sorted particle p.  Reads (x*, lambda) from xin, writes (x* + dp, lambda_i)
// to xout; on the scene's last iteration also the updated velocity into sv.
// Warp-collective like density_lambda_at.
template <bool kPersist, int U, class P, int CH>
__device__ __forceinline__ void delta_at(uint32_t p, bool active, const float4* xin, float4* xout,
                                         const float4* __restrict__ sx,
                                         const float* __restrict__ srho, float4* __restrict__ sv,
                                         int it, const Grid& G, const P& prm,
                                         CoopSmem<CH, false>& sm) {
    constexpr bool kCoop = CoopBlock<P, 32, false, U>::kOn;
    const uint32_t pa = active ? p : 0u;
    const StepConsts& C = prm.at(G.spid, pa);
    const int4 cell = cell_at(G, pa);
    const uint32_t rf = run_flags(G, pa);
    const bool live = active && it < C.iters && !(rf & kCopyBit);
    float4 xi = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    bool walk = live;
    if (live) {
        xi = xin[p];
        // A clean particle with a zero lambda whose 27 cells hold no nonzero
        // lambda in this iteration has only zero terms: no walk.
        if (G.lamnz && cell.w == 0 && xi.w == 0.0f &&
            !neighbourhood_moved<kPersist>(cell, C.grid, G.lamnz, it + 1))
            walk = false;
    }
    // The warp walks cooperatively when every lane is live, even if only
    // some need the walk: the others have only zero terms, which the walk's
    // lambda test leaves out, so they list nothing.
    CoopRow R;
    bool coop = false;
    if constexpr (kCoop) coop = coop_row(live, cell, C.grid, R, scene_at(G, pa));
    if (!live) return;
    float dx = 0.0f, dy = 0.0f, dz = 0.0f;
    auto term = [&](const float4& xj, auto L) {
        float rx, ry, rz, lambda_sum;
        const float r_sq = rel_sq<true>(xi, xj, rx, ry, rz, &lambda_sum);
        // A zero lambda sum adds an exact zero (no s_corr either); the sum,
        // started at +0, never becomes -0, so skipping it keeps every bit.
        if (r_sq < C.cut && lambda_sum != 0.0f) {
            float s_corr = 0.0f;
            if (lambda_sum < -1e-10f && C.scorr_on) {
                float ratio = poly6(r_sq, C) / C.w_dq;
                ratio = (1.0f < ratio) ? 1.0f : ratio;
                float rp = ratio * ratio;
                if (C.corr_n4) rp = rp * rp;
                s_corr = C.neg_corr_k * rp;
            }
            const float c = spiky_coeff(r_sq, C);
            const float a = (lambda_sum + s_corr) * C.mass;
            dx = acc(dx, a * (c * rx), L);
            dy = acc(dy, a * (c * ry), L);
            dz = acc(dz, a * (c * rz), L);
        }
    };
    if constexpr (kCoop) {
        if (coop && __any_sync(0xffffffffu, walk)) {
            coop_walk<CH, false, kPersist, true, false>(
                sm, R, cell.x, xi, xin, C.cut, C.grid, G.off,
                [](uint32_t) { return float4{}; },
                [&](const float4& xj, const float4&) { term(xj, One{}); },
                [&](const float4& xj, const float4&, uint32_t L) { term(xj, L); });
        }
    }
    if (walk && !coop)
        for_each_candidate_runs<U, std::is_same<P, OneScene>::value>(
            cell, G, C, [&](uint32_t q) { term(ld_step<kPersist>(xin + q), One{}); },
            [&](uint32_t q, uint32_t L) { term(ld_step<kPersist>(xin + q), Many{L}); });
    if (G.bg.spos && xi.w != 0.0f) {
        // Two-way coupling: the boundary's share of the position correction,
        // lambda_i (rho0 psi_b) grad W, after the fluid terms (zero when
        // lambda_i is).
        for_each_candidate<4>(boundary_cell(G, p, cell), G.bg.off, G.bg.kpos, G.bg.bend,
                              G.bg.btab, C, [&](uint32_t q) {
                                  const float4 b = __ldg(G.bg.spos + q);
                                  const float rx = xi.x - b.x, ry = xi.y - b.y, rz = xi.z - b.z;
                                  const float r_sq = sqn(rx, ry, rz);
                                  if (r_sq < C.cut) {
                                      const float c = spiky_coeff(r_sq, C);
                                      const float a = xi.w * (C.rho0 * b.w);
                                      dx += a * (c * rx);
                                      dy += a * (c * ry);
                                      dz += a * (c * rz);
                                  }
                              });
    }
    const float px = xi.x + dx * C.inv_rho0;
    const float py = xi.y + dy * C.inv_rho0;
    const float pz = xi.z + dz * C.inv_rho0;
    xout[p] = make_float4(px, py, pz, xi.w);
    if (G.moved && (__float_as_uint(px) != __float_as_uint(xi.x) ||
                    __float_as_uint(py) != __float_as_uint(xi.y) ||
                    __float_as_uint(pz) != __float_as_uint(xi.z)))
        G.moved[slot_of(cell.x, cell.y, cell.z, C.grid)] = (uint32_t)it + 1u;
    float4 vu = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (it == C.iters - 1) sv[p] = vu = update_velocity(px, py, pz, sx[p], srho[p], C);
    for (uint32_t m = p + 1, e = run_end(G, p, rf); m < e; ++m) {
        xout[m] = make_float4(px, py, pz, xi.w);
        if (it == C.iters - 1) sv[m] = vu;
    }
}

template <int BS, class P, int U = 4>
__global__ void __launch_bounds__(BS, kPassMinBlocks<BS>)
k_delta(const float4* __restrict__ xin, float4* __restrict__ xout, const float4* __restrict__ sx,
        const float* __restrict__ srho, float4* __restrict__ sv, int it, int n, const Grid G,
        const P prm) {
    using B = CoopBlock<P, BS, false, U>;
    __shared__ typename B::Smem sm[B::kWarps];
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    delta_at<false, U>(p, p < (uint32_t)n, xin, xout, sx, srho, sv, it, G, prm,
                       sm[B::kOn ? threadIdx.x >> 5 : 0]);
}

// ---------------------------------------------------------------------------
// Persistent Jacobi loop: all iterations of a step in one cooperative launch.
// Every thread keeps the same particles (grid stride) in both passes, and the
// grid meets at a barrier after each pass.

// Grid barrier for a cooperative launch (all blocks resident).  `count` must
// be 0 when the launch starts.  Every wait is bounded: after kBarrierSpins
// polls or kBarrierNs of global time a block records bit 4 in *err and the
// loop returns, so a barrier that cannot complete ends the launch instead of
// hanging it.
struct GridSync {
    unsigned int* count;
    unsigned int* gen;
    uint32_t* err;
};

constexpr uint32_t kBarrierSpins = 1u << 24;
constexpr unsigned long long kBarrierNs = 10ull * 1000 * 1000 * 1000;

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool grid_sync(const GridSync& S) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        const unsigned int g = *(volatile unsigned int*)S.gen;
        __threadfence();  // this block's writes before its arrival
        if (atomicAdd(S.count, 1u) == gridDim.x - 1u) {
            atomicExch(S.count, 0u);
            __threadfence();
            atomicAdd(S.gen, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            for (uint32_t k = 0; *(volatile unsigned int*)S.gen == g; ++k) {
                if (k > kBarrierSpins || global_ns() - t0 > kBarrierNs) {
                    atomicOr(S.err, 4u);
                    ok = 0;
                    break;
                }
                __nanosleep(128);
            }
        }
        __threadfence();  // the other blocks' writes before this block's reads
    }
    __syncthreads();
    return ok != 0;
}

template <class P>
__global__ void __launch_bounds__(kBlock)
k_iterate(float4* xa, float4* xb, float* __restrict__ srho, const float4* __restrict__ sx,
          float4* __restrict__ sv, int max_iters, int n, const Grid G, const P prm,
          const GridSync S) {
    using B = CoopBlock<P, kBlock, false, 4>;
    __shared__ typename B::Smem sm[B::kWarps];
    const uint32_t stride = gridDim.x * blockDim.x;
    // The warp strides as a whole, so that its lanes meet in every
    // warp-collective pass call.
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t w0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
    auto& my = sm[B::kOn ? threadIdx.x >> 5 : 0];
    for (int it = 0; it < max_iters; ++it) {
        for (uint32_t pw = w0; pw < (uint32_t)n; pw += stride)
            density_lambda_at<true, 4>(pw + lane, pw + lane < (uint32_t)n, xa, xb, srho, it, G,
                                       prm, my);
        if (!grid_sync(S)) return;
        for (uint32_t pw = w0; pw < (uint32_t)n; pw += stride)
            delta_at<true, 4>(pw + lane, pw + lane < (uint32_t)n, xb, xa, sx, srho, sv, it, G,
                              prm, my);
        if (it + 1 < max_iters && !grid_sync(S)) return;
    }
}

// Velocity update alone, for scenes with solver_iterations == 0.
template <int BS, class P>
__global__ void __launch_bounds__(BS)
k_velocity(const float4* __restrict__ xin, const float4* __restrict__ sx, const float* __restrict__ srho,
           float4* __restrict__ sv, int n, const Grid G, const P prm) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (uint32_t)n) return;
    const StepConsts& C = prm.at(G.spid, p);
    if (C.iters > 0) return;
    const float4 xi = xin[p];
    sv[p] = update_velocity(xi.x, xi.y, xi.z, sx[p], srho[p], C);
}

// Domain clamp + commit (pbf_solver.cpp:102-126), scattered to particle order.
__device__ __forceinline__ void commit(uint32_t p, float px, float py, float pz, float vx, float vy,
                                       float vz, float lam, const float4* __restrict__ sx,
                                       const float* __restrict__ srho, const StateRef& R, int n,
                                       const StepConsts& C) {
    if (C.clamp) {
        if (px < C.lo[0]) { px = C.lo[0]; vx = 0.0f; } else if (px > C.hi[0]) { px = C.hi[0]; vx = 0.0f; }
        if (py < C.lo[1]) { py = C.lo[1]; vy = 0.0f; } else if (py > C.hi[1]) { py = C.hi[1]; vy = 0.0f; }
        if (pz < C.lo[2]) { pz = C.lo[2]; vz = 0.0f; } else if (pz > C.hi[2]) { pz = C.hi[2]; vz = 0.0f; }
    }
    uint32_t i = __float_as_uint(sx[p].w);
    if (i >= (uint32_t)n) i = 0;
    const uint32_t l = i - R.first;
    if (R.bad && !(isfinite(px) && isfinite(py) && isfinite(pz) && isfinite(vx) && isfinite(vy) &&
                   isfinite(vz)))
        atomicOr(R.bad, 1u);
    R.x[l] = make_float4(px, py, pz, 0.0f);
    R.v[l] = make_float4(vx, vy, vz, 0.0f);
    R.rho[l] = srho[p];
    R.lam[l] = lam;
}

// Boundary friction of two-way steps (StepConsts::bfric), one thread per
// cell-sorted particle after the velocity update and before XSPH:
//   v_i += bfric * sum_b psi_b (v_b - v_i) W(x*_i - x_b),
// an XSPH term against the surface velocity v_b = v_k + w_k x (x_b - p_k) of
// boundary particle b's body k (zero for world-owned particles), over the
// boundary buckets of the particle's cell.  Each thread reads and writes only
// its own velocity.
__global__ void __launch_bounds__(kBlock)
k_boundary_friction(const float4* __restrict__ xin, float4* __restrict__ sv, int n, const Grid G,
                    const StepConsts C) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (uint32_t)n) return;
    const float4 xi = xin[p];
    const float4 vi = sv[p];
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    for_each_candidate<4>(boundary_cell(G, p, cell_at(G, p)), G.bg.off, G.bg.kpos, G.bg.bend,
                          G.bg.btab, C, [&](uint32_t q) {
                              const float4 b = __ldg(G.bg.spos + q);
                              const float rx = xi.x - b.x, ry = xi.y - b.y, rz = xi.z - b.z;
                              const float r_sq = sqn(rx, ry, rz);
                              if (r_sq >= C.h2) return;
                              const int k = __ldg(G.bg.body + __ldg(G.bg.sidx + q));
                              float ux = 0.0f, uy = 0.0f, uz = 0.0f;
                              if (k >= 0 && k < G.bg.nbodies) {
                                  const float4 c = __ldg(G.bg.body_pos + k);
                                  const float4 l = __ldg(G.bg.body_lin + k);
                                  const float4 a = __ldg(G.bg.body_ang + k);
                                  const float dx = b.x - c.x, dy = b.y - c.y, dz = b.z - c.z;
                                  ux = l.x + (a.y * dz - a.z * dy);
                                  uy = l.y + (a.z * dx - a.x * dz);
                                  uz = l.z + (a.x * dy - a.y * dx);
                              }
                              const float w = b.w * poly6(r_sq, C);
                              fx += (ux - vi.x) * w;
                              fy += (uy - vi.y) * w;
                              fz += (uz - vi.z) * w;
                          });
    sv[p] = make_float4(vi.x + C.bfric * fx, vi.y + C.bfric * fy, vi.z + C.bfric * fz, vi.w);
}

// apply_xsph_viscosity (pbf_solver.cpp:225-250) + commit, no vorticity.
// With skip_vort set, scenes with vorticity are left to the vorticity pair.
template <int BS, class P, int U = 4>
__global__ void __launch_bounds__(BS, kPassMinBlocks<BS>)
k_xsph_commit(const float4* __restrict__ xin, const float4* __restrict__ sv, const float4* __restrict__ sx,
              const float* __restrict__ srho, int n, int skip_vort, const Grid G, const P prm) {
    using B = CoopBlock<P, BS, true, U>;
    __shared__ typename B::Smem sm[B::kWarps];
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = p < (uint32_t)n;
    const uint32_t pa = active ? p : 0u;
    const StepConsts& C = prm.at(G.spid, pa);
    const int4 cell = cell_at(G, pa);
    const uint32_t rf = run_flags(G, pa);
    const bool live = active && !(skip_vort && C.vort_on) && !(rf & kCopyBit);
    CoopRow R;
    bool coop = false;
    if constexpr (B::kOn) coop = coop_row(live && C.xsph_on, cell, C.grid, R, scene_at(G, pa));
    if (!live) return;
    const float4 xi = xin[p];
    const float4 vi = sv[p];
    float vx = vi.x, vy = vi.y, vz = vi.z;
    if (C.xsph_on) {
        float cx = 0.0f, cy = 0.0f, cz = 0.0f;
        auto term = [&](const float4& xj, const float4& vj, auto L) {
            float rx, ry, rz;
            const float r_sq = rel_sq(xi, xj, rx, ry, rz);
            if (r_sq < C.h2) {
                const float w = poly6(r_sq, C);
                cx = acc(cx, vj.w * (vj.x - vi.x) * w, L);
                cy = acc(cy, vj.w * (vj.y - vi.y) * w, L);
                cz = acc(cz, vj.w * (vj.z - vi.z) * w, L);
            }
        };
        if constexpr (B::kOn) {
            if (coop)
                coop_walk<coop_chunk(BS), true, false, false, true>(
                    sm[threadIdx.x >> 5], R, cell.x, xi, xin, C.h2, C.grid, G.off,
                    [&](uint32_t q) { return __ldg(sv + q); },
                    [&](const float4& xj, const float4& vj) { term(xj, vj, One{}); },
                    [&](const float4& xj, const float4& vj, uint32_t L) { term(xj, vj, L); });
        }
        if (!coop) {
            auto one = [&](uint32_t q, auto L) {
                const float4 xj = __ldg(xin + q);
                float rx, ry, rz;
                if (rel_sq(xi, xj, rx, ry, rz) < C.h2) term(xj, __ldg(sv + q), L);
            };
            for_each_candidate_runs<U, false>(
                cell, G, C, [&](uint32_t q) { one(q, One{}); },
                [&](uint32_t q, uint32_t L) { one(q, L); });
        }
        vx = vi.x + C.xsph_c * cx;
        vy = vi.y + C.xsph_c * cy;
        vz = vi.z + C.xsph_c * cz;
    }
    for (uint32_t m = p, e = run_end(G, p, rf); m < e; ++m)
        commit(m, xi.x, xi.y, xi.z, vx, vy, vz, xi.w, sx, srho, prm.state(G.spid, m), n, C);
}

// XSPH correction + vorticity omega in one candidate pass (vorticity path).
// Writes the post-XSPH velocity to sv2 and (omega, |omega|) to som, with
//   omega_i = sum_j (m/rho_j') spiky_grad(x*_i - x*_j) x (v_j - v_i),
// the SPH curl (Macklin & Mueller 2013, section 5, with its volume factor).
template <int BS, class P, int U = 4>
__global__ void __launch_bounds__(BS, kPassMinBlocks<BS>)
k_xsph_omega(const float4* __restrict__ xin, const float4* __restrict__ sv, float4* __restrict__ sv2,
             float4* __restrict__ som, int n, const Grid G, const P prm) {
    using B = CoopBlock<P, BS, true, U>;
    __shared__ typename B::Smem sm[B::kWarps];
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = p < (uint32_t)n;
    const uint32_t pa = active ? p : 0u;
    const StepConsts& C = prm.at(G.spid, pa);
    const int4 cell = cell_at(G, pa);
    const uint32_t rf = run_flags(G, pa);
    const bool live = active && C.vort_on && !(rf & kCopyBit);
    CoopRow R;
    bool coop = false;
    if constexpr (B::kOn) coop = coop_row(live, cell, C.grid, R, scene_at(G, pa));
    if (!live) return;
    const float4 xi = xin[p];
    const float4 vi = sv[p];
    float cx = 0.0f, cy = 0.0f, cz = 0.0f, wx = 0.0f, wy = 0.0f, wz = 0.0f;
    auto term = [&](const float4& xj, const float4& vj, auto L) {
        float rx, ry, rz;
        const float r_sq = rel_sq(xi, xj, rx, ry, rz);
        if (r_sq < C.cut) {
            const float ux = vj.x - vi.x;
            const float uy = vj.y - vi.y;
            const float uz = vj.z - vi.z;
            const float w = poly6(r_sq, C);
            cx = acc(cx, vj.w * ux * w, L);
            cy = acc(cy, vj.w * uy * w, L);
            cz = acc(cz, vj.w * uz * w, L);
            const float c = spiky_coeff(r_sq, C);
            const float gx = c * rx, gy = c * ry, gz = c * rz;
            wx = acc(wx, vj.w * (gy * uz - gz * uy), L);
            wy = acc(wy, vj.w * (gz * ux - gx * uz), L);
            wz = acc(wz, vj.w * (gx * uy - gy * ux), L);
        }
    };
    if constexpr (B::kOn) {
        if (coop)
            coop_walk<coop_chunk(BS), true, false, false, true>(
                sm[threadIdx.x >> 5], R, cell.x, xi, xin, C.cut, C.grid, G.off,
                [&](uint32_t q) { return __ldg(sv + q); },
                [&](const float4& xj, const float4& vj) { term(xj, vj, One{}); },
                [&](const float4& xj, const float4& vj, uint32_t L) { term(xj, vj, L); });
    }
    if (!coop) {
        auto one = [&](uint32_t q, auto L) {
            const float4 xj = __ldg(xin + q);
            float rx, ry, rz;
            if (rel_sq(xi, xj, rx, ry, rz) < C.cut) term(xj, __ldg(sv + q), L);
        };
        for_each_candidate_runs<U, false>(
            cell, G, C, [&](uint32_t q) { one(q, One{}); },
            [&](uint32_t q, uint32_t L) { one(q, L); });
    }
    float vx = vi.x, vy = vi.y, vz = vi.z;
    if (C.xsph_on) {
        vx = vi.x + C.xsph_c * cx;
        vy = vi.y + C.xsph_c * cy;
        vz = vi.z + C.xsph_c * cz;
    }
    const float4 o = make_float4(wx, wy, wz, sqrtf(sqn(wx, wy, wz)));
    for (uint32_t m = p, e = run_end(G, p, rf); m < e; ++m) {
        sv2[m] = make_float4(vx, vy, vz, 0.0f);
        som[m] = o;
    }
}

// Vorticity confinement (Macklin & Mueller 2013, section 5) + commit:
//   eta_i = sum_j (m/rho_j') (|omega_j| - |omega_i|) spiky_grad(x*_i - x*_j),
//   N = eta / |eta|,  v += dt * eps * (N x omega_i).
template <int BS, class P, int U = 4>
__global__ void __launch_bounds__(BS, kPassMinBlocks<BS>)
k_vorticity_commit(const float4* __restrict__ xin, const float4* __restrict__ sv,
                   const float4* __restrict__ sv2, const float4* __restrict__ som,
                   const float4* __restrict__ sx, const float* __restrict__ srho, int n,
                   const Grid G, const P prm) {
    using B = CoopBlock<P, BS, true, U>;
    __shared__ typename B::Smem sm[B::kWarps];
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = p < (uint32_t)n;
    const uint32_t pa = active ? p : 0u;
    const StepConsts& C = prm.at(G.spid, pa);
    const int4 cell = cell_at(G, pa);
    const uint32_t rf = run_flags(G, pa);
    const bool live = active && C.vort_on && !(rf & kCopyBit);
    CoopRow R;
    bool coop = false;
    if constexpr (B::kOn) coop = coop_row(live, cell, C.grid, R, scene_at(G, pa));
    if (!live) return;
    const float4 xi = xin[p];
    const float4 wi = som[p];
    float ex = 0.0f, ey = 0.0f, ez = 0.0f;
    // e = (m / rho_j', |omega_j|) of the candidate.
    auto term = [&](const float4& xj, const float4& e, auto L) {
        float rx, ry, rz;
        const float r_sq = rel_sq(xi, xj, rx, ry, rz);
        if (r_sq < C.cut) {
            const float c = spiky_coeff(r_sq, C);
            const float a = e.x * (e.y - wi.w);
            ex = acc(ex, a * (c * rx), L);
            ey = acc(ey, a * (c * ry), L);
            ez = acc(ez, a * (c * rz), L);
        }
    };
    if constexpr (B::kOn) {
        if (coop)
            coop_walk<coop_chunk(BS), true, false, false, true>(
                sm[threadIdx.x >> 5], R, cell.x, xi, xin, C.cut, C.grid, G.off,
                [&](uint32_t q) {
                    return make_float4(__ldg(sv + q).w, __ldg(som + q).w, 0.0f, 0.0f);
                },
                [&](const float4& xj, const float4& e) { term(xj, e, One{}); },
                [&](const float4& xj, const float4& e, uint32_t L) { term(xj, e, L); });
    }
    if (!coop) {
        auto one = [&](uint32_t q, auto L) {
            const float4 xj = __ldg(xin + q);
            float rx, ry, rz;
            if (rel_sq(xi, xj, rx, ry, rz) < C.cut)
                term(xj, make_float4(__ldg(sv + q).w, __ldg(som + q).w, 0.0f, 0.0f), L);
        };
        for_each_candidate_runs<U, false>(
            cell, G, C, [&](uint32_t q) { one(q, One{}); },
            [&](uint32_t q, uint32_t L) { one(q, L); });
    }
    const float el = sqrtf(sqn(ex, ey, ez));
    float nx = 0.0f, ny = 0.0f, nz = 0.0f;
    if (el > 1e-9f) {
        nx = ex / el;
        ny = ey / el;
        nz = ez / el;
    }
    const float fx = ny * wi.z - nz * wi.y;
    const float fy = nz * wi.x - nx * wi.z;
    const float fz = nx * wi.y - ny * wi.x;
    const float4 vb = sv2[p];
    const float vx = vb.x + C.vort_scale * fx;
    const float vy = vb.y + C.vort_scale * fy;
    const float vz = vb.z + C.vort_scale * fz;
    for (uint32_t m = p, e = run_end(G, p, rf); m < e; ++m)
        commit(m, xi.x, xi.y, xi.z, vx, vy, vz, xi.w, sx, srho, prm.state(G.spid, m), n, C);
}

// ---------------------------------------------------------------------------
// Parity probes: cell coordinates and in-radius neighbour lists of x*.

__global__ void __launch_bounds__(kBlock)
k_debug_cells(const float4* __restrict__ x, const float4* __restrict__ v, int* __restrict__ cells3,
              const StepConsts C) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C.n) return;
    float px, py, pz;
    predict(x[i], v[i], C, px, py, pz);
    int cx, cy, cz;
    cell_of(px, py, pz, C.inv_cell, cx, cy, cz);
    cells3[3 * i] = cx;
    cells3[3 * i + 1] = cy;
    cells3[3 * i + 2] = cz;
}

// fill == 0: cnt[i] = number of in-radius candidates j != i of particle i;
// fill == 1: write them (particle indices, candidate order) at out[offs[i]..].
__global__ void __launch_bounds__(kBlock)
k_debug_neighbors(const float4* __restrict__ xin, const float4* __restrict__ sx,
                  long long* __restrict__ cnt, const long long* __restrict__ offs,
                  int* __restrict__ out, long long cap, int fill, const Grid G,
                  const StepConsts C) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (uint32_t)C.n) return;
    const float4 xi = xin[p];
    const uint32_t i = __float_as_uint(sx[p].w);
    long long k = fill ? offs[i] : 0;
    for_each_candidate(cell_at(G, p), G.off, G.kpos, G.bend, G.btab, C, [&](uint32_t q) {
        if (q == p) return;
        const float4 xj = xin[q];
        if (sqn(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z) < C.h2) {
            if (fill && k < cap) out[k] = (int)__float_as_uint(sx[q].w);
            ++k;
        }
    });
    if (!fill) cnt[i] = k;
}

// ---------------------------------------------------------------------------
// Host-side launchers on `stream`.

inline int grid_of(int n, int b) { return (n + b - 1) / b; }

inline Grid grid_view(const StepBuffers& B, const uint32_t* spid = nullptr,
                      const BoundaryGrid& bg = BoundaryGrid{}) {
    return Grid{B.scell, B.sown, B.off, B.kpos, B.bend, B.btab, spid, B.moved, B.lamnz, bg,
                spid ? nullptr : B.dhist, nullptr, B.slot_alias};
}

// predict, sort by cell and by reference key, cell offsets, gather, reference
// buckets, classification: the neighbour structure of one scene's step.
inline cudaError_t enqueue_prefix(const StepBuffers& B, const StepConsts& C, SortScratch& sort,
                                  cudaStream_t st, PhaseMarks* pm = nullptr) {
    const int n = C.n;
    const int nb = grid_of(n, kBlock);
    StepConsts Cs = C;
    Cs.seg_begin = 0;
    Cs.seg_end = (uint32_t)n;
    const OneScene one{Cs, StateRef{B.x, B.v, B.rho, B.lam, 0u, nullptr}};
    const SceneIds none{nullptr, nullptr};
    cudaError_t e = cudaMemsetAsync(B.slot_alias, 0, (size_t)C.grid.nslots, st);
    if (e == cudaSuccess && B.moved) e = cudaMemsetAsync(B.moved, 0, (size_t)C.grid.nslots * 4, st);
    if (e == cudaSuccess && B.lamnz) e = cudaMemsetAsync(B.lamnz, 0, (size_t)C.grid.nslots * 4, st);
    if (e == cudaSuccess && B.dhist) {
        // This step's density-pass counts become the previous step's.
        e = cudaMemcpyAsync(B.dhist, B.dhist + 2 * kWalkHist, 2 * kWalkHist * 4,
                            cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(B.dhist + 2 * kWalkHist, 0, 2 * kWalkHist * 4, st);
    }
    if (e != cudaSuccess) return e;
    if (pm) pm->mark(-1, 0, st);
    k_predict_key<<<nb, kBlock, 0, st>>>(B.keys, B.rkeys, n, none, one);
    if (pm) pm->mark(kPhasePredict, 1, st);
    e = radix_sort_pairs(B.keys, B.skeys, B.sidx, n, C.grid.key_bits, sort, st);
    if (e != cudaSuccess) return e;
    int launches = 2 + (C.grid.key_bits + 7) / 8;
    if (C.hash_compat) {
        e = radix_sort_pairs64(B.rkeys, B.rsorted, B.ridx, n, 64, sort, st);
        if (e != cudaSuccess) return e;
        launches += 9;
    }
    k_offsets<<<grid_of((int)C.grid.nslots + 1, 256), 256, 0, st>>>(B.skeys, n, B.off, C.grid.nslots);
    if (pm) pm->mark(kPhaseGridBuild, launches, st);
    k_gather<<<nb, kBlock, 0, st>>>(B.sidx, B.sx, B.xa, B.srho, B.scell, B.pos_of, B.slot_alias,
                                    B.err, n, none, one);
    if (C.hash_compat) {
        e = enqueue_buckets(B.rsorted, B.ridx, B.pos_of, B.scell, nullptr, B.kpos, B.bend, n, st);
        if (e != cudaSuccess) return e;
        k_classify<<<nb, kBlock, 0, st>>>(B.scell, n, B.scell, B.rsorted, B.kpos, B.bend,
                                          B.slot_alias, B.btab, B.sown, nullptr, one);
    } else {
        e = cudaMemsetAsync(B.sown, 0, (size_t)n * 4, st);
        if (e != cudaSuccess) return e;
    }
    if (pm) pm->mark(kPhaseNeighborQuery, C.hash_compat ? 4 : 1, st);
    return cudaGetLastError();
}

// The constraint, velocity, XSPH, vorticity and commit passes over n
// cell-sorted particles for `max_iters` iterations, with constants from `prm`.
// Scenes with vorticity take the XSPH+omega / vorticity+commit pair
// (any_vort), the others XSPH+commit (any_plain).
// XSPH (+ vorticity) and commit passes with the row loop unrolled U ways.
template <int BS, int U, class P>
inline void enqueue_tail(const StepBuffers& B, const Grid& G, const P& prm, int n, int nb,
                         bool any_vort, bool any_plain, bool xsph_on, cudaStream_t st,
                         PhaseMarks* pm) {
    if (any_vort) {
        k_xsph_omega<BS, P, U><<<nb, BS, 0, st>>>(B.xa, B.sv, B.sv2, B.som, n, G, prm);
        if (pm) pm->mark(kPhaseXsph, 1, st);
        k_vorticity_commit<BS, P, U><<<nb, BS, 0, st>>>(B.xa, B.sv, B.sv2, B.som, B.sx, B.srho,
                                                        n, G, prm);
        if (pm) pm->mark(kPhaseCommit, 1, st);
    }
    if (any_plain) {
        k_xsph_commit<BS, P, U><<<nb, BS, 0, st>>>(B.xa, B.sv, B.sx, B.srho, n,
                                                   any_vort ? 1 : 0, G, prm);
        if (pm) pm->mark(xsph_on ? kPhaseXsph : kPhaseCommit, 1, st);
    }
}

template <int BS, class P>
inline cudaError_t enqueue_passes_bs(const StepBuffers& B, const Grid& G, int n, int max_iters,
                                     bool any_zero_iters, bool any_vort, bool any_plain,
                                     bool xsph_on, const P prm, cudaStream_t st, PhaseMarks* pm,
                                     int persist_blocks, unsigned int* barrier) {
    const int nb = grid_of(n, BS);
    if (persist_blocks > 0 && barrier && max_iters > 0) {
        // The whole Jacobi loop as one cooperative launch.
        cudaError_t e = cudaMemsetAsync(barrier, 0, sizeof(unsigned int), st);
        if (e != cudaSuccess) return e;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)persist_blocks);
        cfg.blockDim = dim3(kBlock);
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        e = cudaLaunchKernelEx(&cfg, k_iterate<P>, B.xa, B.xb, B.srho,
                               static_cast<const float4*>(B.sx), B.sv, max_iters, n, G, prm,
                               GridSync{barrier, barrier + 1, B.err});
        if (e != cudaSuccess) return e;
        if (pm) pm->mark(kPhaseDensity, 1, st);
    } else {
        bool big = false;
        if constexpr (std::is_same<P, OneScene>::value) big = n >= kBigScene;
        for (int it = 0; it < max_iters; ++it) {
            if constexpr (std::is_same<P, OneScene>::value) {
                if (big)
                    k_density_lambda<BS, P, 8><<<nb, BS, 0, st>>>(B.xa, B.xb, B.srho, it, n, G, prm);
                else
                    k_density_lambda<BS, P, 4><<<nb, BS, 0, st>>>(B.xa, B.xb, B.srho, it, n, G, prm);
            } else {
                k_density_lambda<BS, P, 4><<<nb, BS, 0, st>>>(B.xa, B.xb, B.srho, it, n, G, prm);
            }
            if (pm) pm->mark(kPhaseDensity, 1, st);
            if constexpr (std::is_same<P, OneScene>::value) {
                if (big)
                    k_delta<BS, P, 8><<<nb, BS, 0, st>>>(B.xb, B.xa, B.sx, B.srho, B.sv, it, n, G, prm);
                else
                    k_delta<BS, P, 4><<<nb, BS, 0, st>>>(B.xb, B.xa, B.sx, B.srho, B.sv, it, n, G, prm);
            } else {
                k_delta<BS, P, 4><<<nb, BS, 0, st>>>(B.xb, B.xa, B.sx, B.srho, B.sv, it, n, G, prm);
            }
            if (pm) pm->mark(kPhaseDelta, 1, st);
        }
    }
    if (any_zero_iters) {
        k_velocity<BS><<<nb, BS, 0, st>>>(B.xa, B.sx, B.srho, B.sv, n, G, prm);
        if (pm) pm->mark(kPhaseDelta, 1, st);
    }
    if constexpr (std::is_same<P, OneScene>::value) {
        if (G.bg.spos && prm.C.bfric != 0.0f) {
            k_boundary_friction<<<nb, BS, 0, st>>>(B.xa, B.sv, n, G, prm.C);
            if (pm) pm->mark(kPhaseXsph, 1, st);
        }
    }
    if constexpr (std::is_same<P, OneScene>::value) {
        if (n >= kBigScene)
            enqueue_tail<BS, 8>(B, G, prm, n, nb, any_vort, any_plain, xsph_on, st, pm);
        else
            enqueue_tail<BS, 4>(B, G, prm, n, nb, any_vort, any_plain, xsph_on, st, pm);
    } else {
        enqueue_tail<BS, 4>(B, G, prm, n, nb, any_vort, any_plain, xsph_on, st, pm);
    }
    return cudaGetLastError();
}

// The constraint, velocity, XSPH, vorticity and commit passes over n
// cell-sorted particles for `max_iters` iterations, with constants from `prm`.
// Scenes with vorticity take the XSPH+omega / vorticity+commit pair
// (any_vort), the others XSPH+commit (any_plain).  Batches (SceneTable) may
// pick the block size of the neighbour passes (64, 128 or 256 threads); a
// single scene always uses kBlock.
template <class P>
inline cudaError_t enqueue_passes(const StepBuffers& B, const Grid& G, int n, int max_iters,
                                  bool any_zero_iters, bool any_vort, bool any_plain, bool xsph_on,
                                  const P prm, cudaStream_t st, PhaseMarks* pm,
                                  int persist_blocks = 0, unsigned int* barrier = nullptr,
                                  int block = kBlock) {
    if constexpr (std::is_same<P, SceneTable>::value) {
        if (block == 64)
            return enqueue_passes_bs<64>(B, G, n, max_iters, any_zero_iters, any_vort, any_plain,
                                         xsph_on, prm, st, pm, persist_blocks, barrier);
        if (block == 256)
            return enqueue_passes_bs<256>(B, G, n, max_iters, any_zero_iters, any_vort, any_plain,
                                          xsph_on, prm, st, pm, persist_blocks, barrier);
    }
    return enqueue_passes_bs<kBlock>(B, G, n, max_iters, any_zero_iters, any_vort, any_plain,
                                     xsph_on, prm, st, pm, persist_blocks, barrier);
}

inline cudaError_t enqueue_step(const StepBuffers& B, const StepConsts& C, int iters,
                                SortScratch& sort, cudaStream_t st, PhaseMarks* pm = nullptr,
                                const BoundaryGrid* bg = nullptr) {
    const int n = C.n;
    if (n <= 0) return cudaSuccess;
    cudaError_t e = enqueue_prefix(B, C, sort, st, pm);
    if (e != cudaSuccess) return e;
    StepConsts Ci = C;
    Ci.iters = iters;
    BoundaryGrid bgs = bg ? *bg : BoundaryGrid{};
    if (bg) bgs.sx = B.sx;
    Grid G = grid_view(B, nullptr, bgs);
    if (B.segend && n >= kBigScene) {
        // Runs of identical particles: from here on the owner words of the
        // run's later particles carry kCopyBit, which only the passes below
        // understand (they skip those particles).
        k_segments<<<grid_of(n, 256), 256, 0, st>>>(StepState{B.sx, B.xa, B.srho, n}, B.scell,
                                                    C.grid, B.sown, B.slot_alias, B.segend);
        if (pm) pm->mark(kPhaseNeighborQuery, 1, st);
        G.segend = B.segend;
    }
    return enqueue_passes(B, G, n, iters, iters <= 0, C.vort_on != 0,
                          C.vort_on == 0,
                          C.xsph_on != 0, OneScene{Ci, StateRef{B.x, B.v, B.rho, B.lam, 0u, nullptr}}, st,
                          pm);
}

// ---------------------------------------------------------------------------
// Batches of independent scenes: one sort and one launch per phase for all.

// Reorders the key sort stably by scene: rsorted[p] = rtmp[perm[p]],
// ridx[p] = itmp[perm[p]].
__global__ void __launch_bounds__(256)
k_apply_scene_perm(const unsigned long long* __restrict__ rtmp, const uint32_t* __restrict__ itmp,
                   const uint32_t* __restrict__ perm, unsigned long long* __restrict__ rsorted,
                   uint32_t* __restrict__ ridx, int n) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    uint32_t q = perm[p];
    if (q >= (uint32_t)n) q = 0;
    rsorted[p] = rtmp[q];
    ridx[p] = itmp[q];
}

// pid[i] = the scene whose particle range holds batch particle i.
__global__ void __launch_bounds__(256)
k_scene_ids(const uint32_t* __restrict__ firsts, int nscenes, uint32_t* __restrict__ pid, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int a = 0, b = nscenes - 1;  // last s with firsts[s] <= i
    while (a < b) {
        const int m = (a + b + 1) >> 1;
        if (__ldg(firsts + m) <= (uint32_t)i) a = m;
        else b = m - 1;
    }
    pid[i] = (uint32_t)a;
}

__global__ void __launch_bounds__(256)
k_scene_of(const uint32_t* __restrict__ itmp, const uint32_t* __restrict__ pid,
           uint32_t* __restrict__ stmp, int n) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    uint32_t i = itmp[p];
    if (i >= (uint32_t)n) i = 0;
    stmp[p] = pid[i];
}

inline cudaError_t enqueue_batch_step(const StepBuffers& B, const BatchDesc& D, SortScratch& sort,
                                      cudaStream_t st, PhaseMarks* pm = nullptr) {
    const int n = D.n;
    if (n <= 0) return cudaSuccess;
    const int nb = grid_of(n, kBlock);
    const SceneTable tab{D.tab, D.refs};
    const SceneIds ids{D.pid, D.spid};
    cudaError_t e = cudaMemsetAsync(B.slot_alias, 0, (size_t)D.nslots, st);
    if (e == cudaSuccess && B.moved) e = cudaMemsetAsync(B.moved, 0, (size_t)D.nslots * 4, st);
    if (e == cudaSuccess && B.lamnz) e = cudaMemsetAsync(B.lamnz, 0, (size_t)D.nslots * 4, st);
    if (e != cudaSuccess) return e;
    if (pm) pm->mark(-1, 0, st);
    k_scene_ids<<<grid_of(n, 256), 256, 0, st>>>(D.firsts, D.nscenes, D.pid, n);
    k_predict_key<<<nb, kBlock, 0, st>>>(B.keys, B.rkeys, n, ids, tab);
    if (pm) pm->mark(kPhasePredict, 2, st);
    // Cell order: scene-major because every scene owns a slot range.
    e = radix_sort_pairs(B.keys, B.skeys, B.sidx, n, D.key_bits, sort, st);
    if (e != cudaSuccess) return e;
    // Reference buckets per scene: sort by key, then stably by scene.
    e = radix_sort_pairs64(B.rkeys, D.rtmp, D.itmp, n, 64, sort, st);
    if (e != cudaSuccess) return e;
    k_scene_of<<<grid_of(n, 256), 256, 0, st>>>(D.itmp, D.pid, D.stmp, n);
    e = radix_sort_pairs(D.stmp, D.kpid, D.perm, n, D.scene_bits, sort, st);
    if (e != cudaSuccess) return e;
    k_apply_scene_perm<<<grid_of(n, 256), 256, 0, st>>>(D.rtmp, D.itmp, D.perm, B.rsorted, B.ridx,
                                                        n);
    k_offsets<<<grid_of((int)D.nslots + 1, 256), 256, 0, st>>>(B.skeys, n, B.off, D.nslots);
    if (pm) pm->mark(kPhaseGridBuild, 14 + (D.key_bits + 7) / 8 + (D.scene_bits + 7) / 8, st);
    k_gather<<<nb, kBlock, 0, st>>>(B.sidx, B.sx, B.xa, B.srho, B.scell, B.pos_of, B.slot_alias,
                                    B.err, n, ids, tab);
    e = enqueue_buckets(B.rsorted, B.ridx, B.pos_of, B.scell, D.kpid, B.kpos, B.bend, n, st);
    if (e != cudaSuccess) return e;
    k_classify<<<nb, kBlock, 0, st>>>(B.scell, n, B.scell, B.rsorted, B.kpos, B.bend, B.slot_alias,
                                      B.btab, B.sown, D.spid, tab);
    if (pm) pm->mark(kPhaseNeighborQuery, 4, st);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return enqueue_passes(B, grid_view(B, D.spid), n, D.max_iters, D.any_zero_iters, D.any_vort,
                          D.any_plain, D.xsph_on, tab, st, pm, D.persist_blocks, D.barrier,
                          D.block);
}

// Blocks of the persistent Jacobi loop that fit on the device at once.
inline int persist_blocks_max() {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_iterate<SceneTable>, kBlock, 0) !=
        cudaSuccess)
        return 0;
    return sms * per_sm;
}

}  // namespace PBF_NS
}  // namespace pbf
