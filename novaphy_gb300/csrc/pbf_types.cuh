// Plain data shared by the host orchestration and both kernel builds.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace pbf {

// Neighbour grid: cell = h, coordinates floor(x * inv_cell) as in
// SpatialHashGrid::world_to_cell (neighbor_search.cpp:99-105).  Cell (cx,cy,cz)
// lives in slot  wrap(cx-ox) + gx * (wrap(cy-oy) + gy * wrap(cz-oz)),  each
// axis wrapped modulo its extent (>= 4).  Wrapping never merges two cells of
// one 27-neighbourhood, and a wrapped alias is >= 3 cells away, beyond the
// kernel support, so it only adds exact zeros: any origin/extent is correct,
// and a good fit only saves work.
struct GridDesc {
    int ox, oy, oz;
    int gx, gy, gz;
    uint32_t nslots;
    int key_bits;
    uint32_t base;  // first slot of this grid in a batch's global slot space
};

// Per-step constants, all computed on the host in float32 with the
// reference's operation order (pbf_solver.cpp, sph_kernel.h).
struct StepConsts {
    int n;
    float h;         // kernel radius
    float h2;        // h * h                         (sph_kernel.h:25-26)
    float cut;       // smallest r^2 with poly6 == 0 and spiky_grad == 0
    float inv_cell;  // 1.0f / h                      (neighbor_search.cpp:101)
    float mass;
    float rho0;
    float inv_rho0;  // 1.0f / rho0                   (pbf_solver.cpp:149)
    float eps;       // CFM epsilon
    float mr;        // mass * inv_rho0               (pbf_solver.cpp:170)
    float k_poly;    // 315 / (64 pi h^9)             (sph_kernel.h:29)
    float k_spiky;   // -(45 / (pi h^6))              (sph_kernel.h:44)
    float w_dq;      // poly6((dq h)^2, h)            (pbf_solver.cpp:188-189)
    float neg_corr_k;
    int corr_n4;     // corr_n == 4
    int scorr_on;    // w_dq > 1e-10
    float dt, inv_dt, max_speed, max_speed_sq;  // (pbf_solver.cpp:81-83)
    float g[3];
    float xsph_c;
    int xsph_on;     // xsph_viscosity > 0            (pbf_solver.cpp:96)
    float vort_eps;
    float vort_scale;  // dt * vort_eps
    int vort_on;
    int clamp;
    float lo[3], hi[3];  // domain_lower + pr, domain_upper - pr (pbf_solver.cpp:105-107)
    int hash_compat;
    int two_way;         // the boundary enters the constraint (coupled steps)
    float bfric;         // boundary friction coefficient of two-way steps (0: none)
    int iters;           // Jacobi iterations of this scene
    uint32_t seg_begin;  // this scene's range in the key-sorted order of a batch
    uint32_t seg_end;
    GridDesc grid;
};

// The Akinci boundary of a two-way coupled step (pbf_settings.boundary_two_way):
// the reference-bucket index over the boundary's world positions (spos.w =
// psi), each fluid particle's classification against it (own, btab; indexed
// by particle), and the sorted x (sx.w = particle index bits) that maps a
// sorted position to its particle.  All null when the step has none.
struct BoundaryGrid {
    const float4* spos = nullptr;
    const uint32_t* off = nullptr;
    const uint32_t* kpos = nullptr;
    const uint32_t* bend = nullptr;
    const int* own = nullptr;
    const uint32_t* btab = nullptr;
    const float4* sx = nullptr;
    // Boundary friction: the index's sorted-to-original map, each original
    // boundary particle's body, and the bodies' poses and velocities.
    const uint32_t* sidx = nullptr;
    const int* body = nullptr;
    int nbodies = 0;
    const float4* body_pos = nullptr;
    const float4* body_lin = nullptr;
    const float4* body_ang = nullptr;
};

// Device buffers of one step.  Arrays named s* are in sorted (cell) order.
struct StepBuffers {
    float4* x;      // positions, particle order (w unused)
    float4* v;      // velocities, particle order
    float* rho;     // densities, particle order
    float* lam;     // lambdas, particle order
    uint32_t* keys;   // slot per particle, particle order
    uint32_t* skeys;  // sorted slots
    uint32_t* sidx;   // particle index of sorted position p
    uint32_t* off;    // off[s] = first sorted position with slot >= s; nslots+1 entries
    float4* sx;     // x (w = particle index bits)
    float4* xa;     // x* ping (w = lambda)
    float4* xb;     // x* pong
    float4* sv;     // post-update velocity (w = m / rho')
    float4* sv2;    // post-XSPH velocity (vorticity path)
    float4* som;    // vorticity omega (w = |omega|)
    float* srho;    // densities of the last density pass
    int4* scell;    // cell of x* at step start
    // Reference hash buckets (neighbor_search.cpp:14-22) for exact candidate
    // lists where they differ from the plain 27-cell neighbourhood.
    unsigned long long* rkeys;    // reference key per particle, particle order
    unsigned long long* rsorted;  // keys sorted (stable)
    uint32_t* ridx;      // particle of key-sorted position
    uint32_t* pos_of;    // cell-sorted position of each particle
    uint32_t* kpos;      // cell-sorted position of each key-sorted position
    uint32_t* bend;      // at bucket starts: bucket end | impure bit
    uint32_t* btab;      // 27 bucket starts per dirty owner row
    int* sown;           // 0 = clean, else owner row + 1
    unsigned char* slot_alias;  // slot holds a particle from outside the grid box
    // Per slot: 1 + the Jacobi iteration whose delta pass last moved a
    // particle of the slot (0: none in this step).
    uint32_t* moved;
    // Per slot: 1 + the Jacobi iteration whose density pass last left a
    // particle of the slot with a nonzero lambda (0: none in this step).
    uint32_t* lamnz;
    // Per Jacobi iteration (kWalkHist of them): how many cooperative warps
    // of the density pass had a lane with C_i >= 0, and how many ran, in
    // the previous step ([0, 2 kWalkHist)) and in this one (the rest).
    // Single scenes only (null in batches).
    uint32_t* dhist;
    // Per sorted position: for the first particle of a run of particles with
    // bit-identical step state in cell order, one past the run's last; 0
    // elsewhere (see k_segments).  Single scenes only (null in batches).
    uint32_t* segend;
    uint32_t* err;  // device status word
};

constexpr int kWalkHist = 16;

// Phases of one step, named after the reference's PerformanceMonitor scopes
// (pbf_solver.cpp:29-103).  Fused kernels report under the first scope they
// cover: density+lambda under compute_density, delta+apply(+velocity update
// on the last iteration) under compute_delta_position, XSPH(+vorticity omega)
// under xsph_viscosity, vorticity confinement + clamp + commit under
// commit_positions.
enum StepPhase {
    kPhasePredict = 0,
    kPhaseGridBuild = 1,
    kPhaseNeighborQuery = 2,
    kPhaseDensity = 3,
    kPhaseDelta = 4,
    kPhaseXsph = 5,
    kPhaseCommit = 6,
    kNumPhases = 7
};

// Event marks between the launches of one step (profiling only).
struct PhaseMarks {
    static constexpr int kMax = 96;
    cudaEvent_t ev[kMax];
    int phase[kMax];
    int launches[kMax];
    int count = 0;
    // Records the end of a phase that launched `nl` kernels.
    void mark(int ph, int nl, cudaStream_t st) {
        if (count < kMax) {
            cudaEventRecord(ev[count], st);
            phase[count] = ph;
            launches[count] = nl;
            ++count;
        }
    }
};

// Particle-order state of one scene of a batch; batch particle i of the
// scene is the scene's particle i - first.
struct StateRef {
    float4* x;
    float4* v;
    float* rho;
    float* lam;
    uint32_t first;
    uint32_t* bad;  // set to 1 when a committed x or v is not finite (null: no check)
};

// One step of a batch of independent scenes: particle i of the batch belongs
// to scene pid[i]; scenes occupy consecutive particle ranges [firsts[s],
// firsts[s+1]) and consecutive slot ranges of one global cell-slot space.
struct BatchDesc {
    int n;               // particles of all scenes
    int nscenes;
    uint32_t nslots;     // global slot space (sum of the scenes' grids)
    int key_bits;        // bits of a global slot
    int scene_bits;      // bits of a scene id
    int max_iters;       // largest solver_iterations of the batch
    bool any_zero_iters, any_vort, any_plain, xsph_on;
    const StepConsts* tab;  // device tables, one entry per scene
    const StateRef* refs;
    const uint32_t* firsts;    // nscenes + 1 particle offsets
    uint32_t* pid;             // scene of each particle (particle order)
    uint32_t* spid;            // scene of each cell-sorted particle
    uint32_t* kpid;            // scene of each key-sorted particle
    unsigned long long* rtmp;  // key-sorted keys before the scene pass
    uint32_t* itmp;            // key-sorted particles before the scene pass
    uint32_t* perm;            // scene-pass permutation
    uint32_t* stmp;            // scenes of the key-sorted particles before the scene pass
    int persist_blocks;        // > 0: the Jacobi loop as one cooperative launch of this grid
    unsigned int* barrier;     // its grid barrier (count, generation)
    int block;                 // threads per block of the neighbour passes (64, 128, 256)
};

}  // namespace pbf
