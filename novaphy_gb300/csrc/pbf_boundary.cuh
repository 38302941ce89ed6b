// Akinci rigid-fluid coupling on the device (src/fluid/boundary.cpp,
// src/fluid/fluid_world.cpp): boundary world positions, boundary density,
// coupling forces and torques with a serial per-body reduction in boundary
// order, Akinci volumes.  Every neighbour sum walks the reference's hash
// buckets (neighbor_search.cpp:14-49) through a PointIndex.
#pragma once

#include <cstdint>

#include "novaphy_pbf.h"
#include "pbf_types.cuh"
#include "radix_sort.cuh"

namespace pbf {

// The reference's hash grid over one point set, laid out like the step's:
// dense wrapped cell slots (keys -> skeys/sidx, off, slot_alias) for spatial
// order, and the reference keys sorted (rsorted/ridx) for exact buckets.
struct PointIndex {
    int n = 0;
    uint32_t* keys = nullptr;
    uint32_t* skeys = nullptr;
    uint32_t* sidx = nullptr;
    unsigned long long* rkeys = nullptr;
    unsigned long long* rsorted = nullptr;
    uint32_t* ridx = nullptr;
    uint32_t* pos_of = nullptr;
    uint32_t* kpos = nullptr;
    uint32_t* bend = nullptr;
    float4* spos = nullptr;  // sorted positions, w = per-point attribute
    int4* scell = nullptr;
    uint32_t* off = nullptr;            // nslots + 1
    unsigned char* slot_alias = nullptr;  // nslots
};

// Queries against a PointIndex: cell of each query point, dirty owner and
// the 27 bucket starts of dirty owners.
struct QuerySet {
    int4* qcell = nullptr;
    int* qown = nullptr;
    uint32_t* btab = nullptr;  // 27 per query
};

// Builds `I` over pos[0..n) (xyz) with attribute attr[i] (or pos.w when
// attr is null) on stream `st`.
cudaError_t index_build(PointIndex& I, const float4* pos, const float* attr, int n,
                        const StepConsts& C, SortScratch& sort, cudaStream_t st);

// x* = x + (v + g dt) dt of n particles (w = 0): the positions whose cells
// a step sorts by (the predict of k_predict_key, the same operations).
cudaError_t predict_points(const float4* x, const float4* v, int n, float4* out,
                           const StepConsts& C, cudaStream_t st);

// Classifies query points qpos[0..nq) against `I`.
cudaError_t index_classify(const QuerySet& Q, const float4* qpos, int nq, const PointIndex& I,
                           const StepConsts& C, cudaStream_t st);

// x_b = T[body] * local (boundary.cpp:178-192); w carries psi.
cudaError_t boundary_xform(const float4* local, const int* body, int nb, const float4* body_pos,
                           const float4* body_quat, int nbodies, float4* world, cudaStream_t st);

// rho_i += sum_b rho0 psi_b poly6(|x_i - x_b|^2) over boundary buckets
// (fluid_world.cpp:101-123); x and rho in particle order.
cudaError_t boundary_density(const float4* x, int n, const QuerySet& Q, const PointIndex& bidx,
                             float* rho, const StepConsts& C, cudaStream_t st);

// Per-boundary-particle pressure force from the fluid (fluid_world.cpp:
// 136-161); fidx indexes final fluid positions with w = density.
// Fb[b].w = 1 when |F_b|^2 > 1e-20 (the reference's apply threshold).
cudaError_t coupling_forces(const float4* bworld, const int* body, const int* body_dynamic,
                            int nb, int nbodies, const QuerySet& Q, const PointIndex& fidx,
                            float4* Fb, const StepConsts& C, cudaStream_t st);

// force/torque[k] += F_b, (x_b - p_k) x F_b over body k's boundary particles.
// tree = false: one thread per body adds them in ascending b, the reference's
// order (fluid_world.cpp:163-172 + World::apply_force/torque), bit for bit.
// tree = true: a deterministic segmented tree reduction (one block per body,
// fixed pairing), within 2 (m - 1) 2^-24 sum_b |term_b| of the serial sum for
// a body of m terms.
cudaError_t body_reduce(const float4* Fb, const float4* bworld, const int* list_off,
                        const int* list, const float4* body_pos, int nbodies, float* force3,
                        float* torque3, bool tree, cudaStream_t st);

// Rigid step of the bodies with inv_mass > 0 under gravity g and the coupling
// force/torque of the step (force3/torque3 hold the first nforce bodies; the
// others receive none), then the new poses of the first nforce bodies into
// body_pos/body_quat for the next step's boundary positions.  The same float
// operations as the host rigid step (rigid_step.hpp).
cudaError_t rigid_step(pbf_rigid_body* bodies, int nbodies, const float* force3,
                       const float* torque3, int nforce, float gx, float gy, float gz, float dt,
                       float4* body_pos, float4* body_quat, cudaStream_t st);

// World's rigid pipeline with sphere and plane contacts (rigid_world.cuh)
// for one scene's bodies, in place of rigid_step; the same outputs.
// Shapes must have been validated (types, bodies, at most 16 of each).
cudaError_t rigid_world(pbf_rigid_body* bodies, int nbodies, const pbf_rigid_shape* shapes,
                        int nshapes, const pbf_contact_settings& set, const float* force3,
                        const float* torque3, int nforce, float gx, float gy, float gz, float dt,
                        float4* body_pos, float4* body_quat, cudaStream_t st);

// psi_b = 1 / sum_b' poly6 (0 when the sum <= 1e-10), boundary.cpp:152-176.
cudaError_t boundary_volumes(const float4* world, int nb, const QuerySet& Q, const PointIndex& I,
                             float* psi, const StepConsts& C, cudaStream_t st);

}  // namespace pbf
