// Akinci coupling kernels (see pbf_boundary.cuh).  Built with the exact
// arithmetic flags (-fmad=false, IEEE div/sqrt): every expression follows the
// reference's operation order (src/fluid/boundary.cpp, fluid_world.cpp).
#define PBF_FAST 0
#define PBF_NS bnd
#include "pbf_boundary.cuh"
#include "pbf_kernels.cuh"
#include "rigid_step.hpp"
#include "rigid_world.cuh"

namespace pbf {
namespace bnd {

// Cell slot and reference key of points (no prediction).
__global__ void __launch_bounds__(kBlock)
k_ix_keys(const float4* __restrict__ pos, int n, uint32_t* __restrict__ keys,
          unsigned long long* __restrict__ rkeys, const StepConsts C) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    int cx, cy, cz;
    cell_of(p.x, p.y, p.z, C.inv_cell, cx, cy, cz);
    keys[i] = slot_of(cx, cy, cz, C.grid);
    rkeys[i] = ref_hash(cx, cy, cz);
}

__global__ void __launch_bounds__(kBlock)
k_ix_gather(const uint32_t* __restrict__ sidx, const float4* __restrict__ pos,
            const float* __restrict__ attr, int n, float4* __restrict__ spos,
            int4* __restrict__ scell, uint32_t* __restrict__ pos_of,
            unsigned char* __restrict__ slot_alias, const StepConsts C) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    uint32_t i = sidx[p];
    if (i >= (uint32_t)n) i = 0;
    const float4 q = pos[i];
    int cx, cy, cz;
    cell_of(q.x, q.y, q.z, C.inv_cell, cx, cy, cz);
    spos[p] = make_float4(q.x, q.y, q.z, attr ? attr[i] : q.w);
    scell[p] = make_int4(cx, cy, cz, 0);
    pos_of[i] = (uint32_t)p;
    if (!in_grid(cx, cy, cz, C.grid)) slot_alias[slot_of(cx, cy, cz, C.grid)] = 1;
}

__global__ void __launch_bounds__(kBlock)
k_predict_points(const float4* __restrict__ x, const float4* __restrict__ v, int n,
                 float4* __restrict__ out, const StepConsts C) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float px, py, pz;
    predict(x[i], v[i], C, px, py, pz);
    out[i] = make_float4(px, py, pz, 0.0f);
}

__global__ void __launch_bounds__(kBlock)
k_qcells(const float4* __restrict__ qpos, int nq, int4* __restrict__ qcell, const StepConsts C) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const float4 q = qpos[i];
    int cx, cy, cz;
    cell_of(q.x, q.y, q.z, C.inv_cell, cx, cy, cz);
    qcell[i] = make_int4(cx, cy, cz, 0);
}

__device__ __forceinline__ int4 query_cell(const QuerySet& Q, int i) {
    int4 c = Q.qcell[i];
    c.w = Q.qown[i];
    return c;
}

// (p + q * v) for unit quaternion q = (w, x, y, z), in the order of the
// quaternion-vector product t = 2 (q.vec x v); v + w t + q.vec x t.
__device__ __forceinline__ float3 transform_point(const float4 p, const float4 q, const float4 v) {
    float t0 = q.z * v.z - q.w * v.y;
    float t1 = q.w * v.x - q.y * v.z;
    float t2 = q.y * v.y - q.z * v.x;
    t0 = t0 + t0;
    t1 = t1 + t1;
    t2 = t2 + t2;
    const float c0 = q.z * t2 - q.w * t1;
    const float c1 = q.w * t0 - q.y * t2;
    const float c2 = q.y * t1 - q.z * t0;
    const float r0 = (v.x + q.x * t0) + c0;
    const float r1 = (v.y + q.x * t1) + c1;
    const float r2 = (v.z + q.x * t2) + c2;
    return make_float3(p.x + r0, p.y + r1, p.z + r2);
}

__global__ void __launch_bounds__(kBlock)
k_bxform(const float4* __restrict__ local, const int* __restrict__ body, int nb,
         const float4* __restrict__ body_pos, const float4* __restrict__ body_quat, int nbodies,
         float4* __restrict__ world) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const float4 l = local[b];
    const int bi = body[b];
    if (bi >= 0 && bi < nbodies) {
        const float3 w = transform_point(body_pos[bi], body_quat[bi], l);
        world[b] = make_float4(w.x, w.y, w.z, l.w);
    } else {
        world[b] = l;
    }
}

__global__ void __launch_bounds__(kBlock)
k_boundary_density(const float4* __restrict__ x, int n, const QuerySet Q, const PointIndex I,
                   float* __restrict__ rho, const StepConsts C) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 xi = x[i];
    float bd = 0.0f;
    for_each_candidate(query_cell(Q, i), I.off, I.kpos, I.bend, Q.btab, C, [&](uint32_t q) {
        const float4 b = __ldg(I.spos + q);
        const float r_sq = sqn(xi.x - b.x, xi.y - b.y, xi.z - b.z);
        bd += C.rho0 * b.w * poly6(r_sq, C);
    });
    rho[i] += bd;
}

__global__ void __launch_bounds__(kBlock)
k_coupling(const float4* __restrict__ bworld, const int* __restrict__ body,
           const int* __restrict__ body_dynamic, int nb, int nbodies, const QuerySet Q,
           const PointIndex I, float4* __restrict__ Fb, const StepConsts C) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int bi = body[b];
    if (bi < 0 || bi >= nbodies || !body_dynamic[bi]) {
        Fb[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const float4 xb = bworld[b];
    const float psi_b = xb.w;
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    for_each_candidate(query_cell(Q, b), I.off, I.kpos, I.bend, Q.btab, C, [&](uint32_t q) {
        const float4 xf = __ldg(I.spos + q);
        const float rx = xb.x - xf.x;
        const float ry = xb.y - xf.y;
        const float rz = xb.z - xf.z;
        const float r_sq = sqn(rx, ry, rz);
        if (r_sq >= C.h2) return;
        const float rho_f = (xf.w < 1.0f) ? 1.0f : xf.w;  // std::max(rho, 1.0f)
        const float pd = rho_f - C.rho0;
        const float pressure = (0.0f < pd) ? pd : 0.0f;   // std::max(0.0f, rho - rho0)
        const float pc = C.mass * pressure / (rho_f * rho_f);
        const float c = spiky_coeff(r_sq, C);
        const float a = pc * C.rho0 * psi_b;
        fx += a * (c * rx);
        fy += a * (c * ry);
        fz += a * (c * rz);
    });
    Fb[b] = make_float4(fx, fy, fz, sqn(fx, fy, fz) > 1e-20f ? 1.0f : 0.0f);
}

__global__ void k_body_reduce(const float4* __restrict__ Fb, const float4* __restrict__ bworld,
                              const int* __restrict__ list_off, const int* __restrict__ list,
                              const float4* __restrict__ body_pos, int nbodies,
                              float* __restrict__ force3, float* __restrict__ torque3) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nbodies) return;
    float f0 = force3[3 * k], f1 = force3[3 * k + 1], f2 = force3[3 * k + 2];
    float t0 = torque3[3 * k], t1 = torque3[3 * k + 1], t2 = torque3[3 * k + 2];
    const float4 c = body_pos[k];
    for (int j = list_off[k]; j < list_off[k + 1]; ++j) {
        const int b = list[j];
        const float4 F = Fb[b];
        if (F.w == 0.0f) continue;
        f0 += F.x;
        f1 += F.y;
        f2 += F.z;
        const float4 x = bworld[b];
        const float r0 = x.x - c.x, r1 = x.y - c.y, r2 = x.z - c.z;
        t0 += r1 * F.z - r2 * F.y;
        t1 += r2 * F.x - r0 * F.z;
        t2 += r0 * F.y - r1 * F.x;
    }
    force3[3 * k] = f0;
    force3[3 * k + 1] = f1;
    force3[3 * k + 2] = f2;
    torque3[3 * k] = t0;
    torque3[3 * k + 1] = t1;
    torque3[3 * k + 2] = t2;
}

// Segmented tree reduction of the same sums: one block per body.  Thread t
// adds the list entries t, t + kTreeThreads, ... of its body in that order,
// then the block folds its partial sums pairwise (partial[t] += partial[t + s]
// for s = 128, 64, ..., 1), so every run adds the same floats in the same
// order: the result is deterministic, whatever the schedule.  It rounds
// differently from the serial sum above (the reference's order), by at most
// 2 (m - 1) 2^-24 sum_b |term_b| per component over a body's m terms.
constexpr int kTreeThreads = 256;

__global__ void __launch_bounds__(kTreeThreads)
k_body_reduce_tree(const float4* __restrict__ Fb, const float4* __restrict__ bworld,
                   const int* __restrict__ list_off, const int* __restrict__ list,
                   const float4* __restrict__ body_pos, int nbodies, float* __restrict__ force3,
                   float* __restrict__ torque3) {
    __shared__ float part[6][kTreeThreads];
    const int k = blockIdx.x;
    if (k >= nbodies) return;
    const int t = threadIdx.x;
    const float4 c = body_pos[k];
    float a[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    const int j1 = list_off[k + 1];
    for (int j = list_off[k] + t; j < j1; j += kTreeThreads) {
        const int b = __ldg(list + j);
        const float4 F = __ldg(Fb + b);
        if (F.w == 0.0f) continue;
        const float4 x = __ldg(bworld + b);
        const float r0 = x.x - c.x, r1 = x.y - c.y, r2 = x.z - c.z;
        a[0] += F.x;
        a[1] += F.y;
        a[2] += F.z;
        a[3] += r1 * F.z - r2 * F.y;
        a[4] += r2 * F.x - r0 * F.z;
        a[5] += r0 * F.y - r1 * F.x;
    }
#pragma unroll
    for (int d = 0; d < 6; ++d) part[d][t] = a[d];
    __syncthreads();
#pragma unroll 1
    for (int s = kTreeThreads / 2; s > 0; s >>= 1) {
        if (t < s) {
#pragma unroll
            for (int d = 0; d < 6; ++d) part[d][t] += part[d][t + s];
        }
        __syncthreads();
    }
    if (t < 3) {
        force3[3 * k + t] += part[t][0];
        torque3[3 * k + t] += part[3 + t][0];
    }
}

// One thread per body (rigid_step.hpp on the device).
__global__ void k_rigid_step(pbf_rigid_body* __restrict__ bodies, int nbodies,
                             const float* __restrict__ force3, const float* __restrict__ torque3,
                             int nforce, float gx, float gy, float gz, float dt,
                             float4* __restrict__ body_pos, float4* __restrict__ body_quat) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nbodies) return;
    pbf_rigid_body r = bodies[k];
    if (r.inv_mass > 0.0f) {
        const float g[3] = {gx, gy, gz};
        float f[3] = {0.0f, 0.0f, 0.0f}, t[3] = {0.0f, 0.0f, 0.0f};
        if (k < nforce)
            for (int d = 0; d < 3; ++d) {
                f[d] = force3[3 * k + d];
                t[d] = torque3[3 * k + d];
            }
        pbf_rigid::integrate_velocity(r.lin_vel, r.ang_vel, g, f, r.inv_mass, r.inv_inertia, t, dt);
        pbf_rigid::integrate_position(r.pos, r.quat, r.lin_vel, r.ang_vel, dt);
        bodies[k] = r;
    }
    if (k < nforce) {
        body_pos[k] = make_float4(r.pos[0], r.pos[1], r.pos[2], 0.0f);
        body_quat[k] = make_float4(r.quat[0], r.quat[1], r.quat[2], r.quat[3]);
    }
}

// World's rigid pipeline for one scene's bodies and shapes (rigid_world.cuh),
// in shared memory by one thread; then the new poses of the first nforce
// bodies into body_pos/body_quat, as k_rigid_step.
__global__ void __launch_bounds__(32)
k_rigid_world(pbf_rigid_body* __restrict__ bodies, int nbodies,
              const pbf_rigid_shape* __restrict__ shapes, int nshapes, pbf_contact_settings set,
              const float* __restrict__ force3, const float* __restrict__ torque3, int nforce,
              float gx, float gy, float gz, float dt, float4* __restrict__ body_pos,
              float4* __restrict__ body_quat) {
    __shared__ rw::World W;
    __shared__ pbf_rigid_body B[rw::kMaxShapes];
    __shared__ pbf_rigid_shape S[rw::kMaxShapes];
    if (threadIdx.x != 0 || nbodies > rw::kMaxShapes || nshapes > rw::kMaxShapes) return;
    for (int k = 0; k < nbodies; ++k) B[k] = bodies[k];
    for (int k = 0; k < nshapes; ++k) S[k] = shapes[k];
    const float g[3] = {gx, gy, gz};
    if (rw::world_step(W, B, nbodies, S, nshapes, set, force3, torque3, nforce, g, dt)) return;
    for (int k = 0; k < nbodies; ++k) bodies[k] = B[k];
    for (int k = 0; k < nforce && k < nbodies; ++k) {
        body_pos[k] = make_float4(B[k].pos[0], B[k].pos[1], B[k].pos[2], 0.0f);
        body_quat[k] = make_float4(B[k].quat[0], B[k].quat[1], B[k].quat[2], B[k].quat[3]);
    }
}

__global__ void __launch_bounds__(kBlock)
k_volumes(const float4* __restrict__ world, int nb, const QuerySet Q, const PointIndex I,
          float* __restrict__ psi, const StepConsts C) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const float4 xb = world[b];
    float sum_w = 0.0f;
    for_each_candidate(query_cell(Q, b), I.off, I.kpos, I.bend, Q.btab, C, [&](uint32_t q) {
        const float4 xj = __ldg(I.spos + q);
        sum_w += poly6(sqn(xb.x - xj.x, xb.y - xj.y, xb.z - xj.z), C);
    });
    psi[b] = (sum_w > 1e-10f) ? 1.0f / sum_w : 0.0f;
}

}  // namespace bnd

cudaError_t index_build(PointIndex& I, const float4* pos, const float* attr, int n,
                        const StepConsts& C, SortScratch& sort, cudaStream_t st) {
    using namespace bnd;
    I.n = n;
    if (n <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(I.slot_alias, 0, (size_t)C.grid.nslots, st);
    if (e != cudaSuccess) return e;
    const int nb = grid_of(n, kBlock);
    k_ix_keys<<<nb, kBlock, 0, st>>>(pos, n, I.keys, I.rkeys, C);
    e = radix_sort_pairs(I.keys, I.skeys, I.sidx, n, C.grid.key_bits, sort, st);
    if (e != cudaSuccess) return e;
    e = radix_sort_pairs64(I.rkeys, I.rsorted, I.ridx, n, 64, sort, st);
    if (e != cudaSuccess) return e;
    k_offsets<<<grid_of((int)C.grid.nslots + 1, 256), 256, 0, st>>>(I.skeys, n, I.off, C.grid.nslots);
    k_ix_gather<<<nb, kBlock, 0, st>>>(I.sidx, pos, attr, n, I.spos, I.scell, I.pos_of,
                                       I.slot_alias, C);
    return enqueue_buckets(I.rsorted, I.ridx, I.pos_of, I.scell, nullptr, I.kpos, I.bend, n, st);
}

cudaError_t predict_points(const float4* x, const float4* v, int n, float4* out,
                           const StepConsts& C, cudaStream_t st) {
    using namespace bnd;
    if (n <= 0) return cudaSuccess;
    k_predict_points<<<grid_of(n, kBlock), kBlock, 0, st>>>(x, v, n, out, C);
    return cudaGetLastError();
}

cudaError_t index_classify(const QuerySet& Q, const float4* qpos, int nq, const PointIndex& I,
                           const StepConsts& C, cudaStream_t st) {
    using namespace bnd;
    if (nq <= 0) return cudaSuccess;
    k_qcells<<<grid_of(nq, kBlock), kBlock, 0, st>>>(qpos, nq, Q.qcell, C);
    if (I.n <= 0) {
        // Nothing to find: every neighbour bucket is empty.
        return cudaMemsetAsync(Q.qown, 0, (size_t)nq * sizeof(int), st);
    }
    StepConsts Cs = C;
    Cs.seg_begin = 0;
    Cs.seg_end = (uint32_t)I.n;
    Cs.hash_compat = 1;  // the coupling queries always follow the reference buckets
    k_classify<<<grid_of(nq, kBlock), kBlock, 0, st>>>(Q.qcell, nq, I.scell, I.rsorted, I.kpos,
                                                        I.bend, I.slot_alias, Q.btab, Q.qown,
                                                        nullptr, OneScene{Cs, StateRef{}});
    return cudaGetLastError();
}

cudaError_t boundary_xform(const float4* local, const int* body, int nb, const float4* body_pos,
                           const float4* body_quat, int nbodies, float4* world, cudaStream_t st) {
    using namespace bnd;
    if (nb <= 0) return cudaSuccess;
    k_bxform<<<grid_of(nb, kBlock), kBlock, 0, st>>>(local, body, nb, body_pos, body_quat, nbodies,
                                                     world);
    return cudaGetLastError();
}

cudaError_t boundary_density(const float4* x, int n, const QuerySet& Q, const PointIndex& bidx,
                             float* rho, const StepConsts& C, cudaStream_t st) {
    using namespace bnd;
    if (n <= 0 || bidx.n <= 0) return cudaSuccess;
    k_boundary_density<<<grid_of(n, kBlock), kBlock, 0, st>>>(x, n, Q, bidx, rho, C);
    return cudaGetLastError();
}

cudaError_t coupling_forces(const float4* bworld, const int* body, const int* body_dynamic,
                            int nb, int nbodies, const QuerySet& Q, const PointIndex& fidx,
                            float4* Fb, const StepConsts& C, cudaStream_t st) {
    using namespace bnd;
    if (nb <= 0) return cudaSuccess;
    if (fidx.n <= 0) return cudaMemsetAsync(Fb, 0, (size_t)nb * sizeof(float4), st);
    k_coupling<<<grid_of(nb, kBlock), kBlock, 0, st>>>(bworld, body, body_dynamic, nb, nbodies, Q,
                                                       fidx, Fb, C);
    return cudaGetLastError();
}

cudaError_t body_reduce(const float4* Fb, const float4* bworld, const int* list_off,
                        const int* list, const float4* body_pos, int nbodies, float* force3,
                        float* torque3, bool tree, cudaStream_t st) {
    using namespace bnd;
    if (nbodies <= 0) return cudaSuccess;
    if (tree)
        k_body_reduce_tree<<<nbodies, kTreeThreads, 0, st>>>(Fb, bworld, list_off, list, body_pos,
                                                             nbodies, force3, torque3);
    else
        k_body_reduce<<<grid_of(nbodies, 32), 32, 0, st>>>(Fb, bworld, list_off, list, body_pos,
                                                           nbodies, force3, torque3);
    return cudaGetLastError();
}

cudaError_t rigid_world(pbf_rigid_body* bodies, int nbodies, const pbf_rigid_shape* shapes,
                        int nshapes, const pbf_contact_settings& set, const float* force3,
                        const float* torque3, int nforce, float gx, float gy, float gz, float dt,
                        float4* body_pos, float4* body_quat, cudaStream_t st) {
    using namespace bnd;
    if (nbodies <= 0) return cudaSuccess;
    k_rigid_world<<<1, 32, 0, st>>>(bodies, nbodies, shapes, nshapes, set, force3, torque3, nforce,
                                    gx, gy, gz, dt, body_pos, body_quat);
    return cudaGetLastError();
}

cudaError_t rigid_step(pbf_rigid_body* bodies, int nbodies, const float* force3,
                       const float* torque3, int nforce, float gx, float gy, float gz, float dt,
                       float4* body_pos, float4* body_quat, cudaStream_t st) {
    using namespace bnd;
    if (nbodies <= 0) return cudaSuccess;
    k_rigid_step<<<grid_of(nbodies, 32), 32, 0, st>>>(bodies, nbodies, force3, torque3, nforce, gx,
                                                      gy, gz, dt, body_pos, body_quat);
    return cudaGetLastError();
}

cudaError_t boundary_volumes(const float4* world, int nb, const QuerySet& Q, const PointIndex& I,
                             float* psi, const StepConsts& C, cudaStream_t st) {
    using namespace bnd;
    if (nb <= 0) return cudaSuccess;
    k_volumes<<<grid_of(nb, kBlock), kBlock, 0, st>>>(world, nb, Q, I, psi, C);
    return cudaGetLastError();
}

}  // namespace pbf
