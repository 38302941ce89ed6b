// Rigid contacts of a served coupled scene on the device: World's rigid
// pipeline (src/sim/world.cpp:30-182 with sleep off) for bodies whose shapes
// are spheres and planes, run by one thread per scene:
//   symplectic Euler velocity update (src/dynamics/integrator.cpp:20-60),
//   shape boxes and the broad phase (every pair of overlapping boxes, closed
//   intervals, less pairs of two fixed shapes, in (lower, higher) order),
//   sphere-sphere and sphere-plane contacts (src/collision/narrowphase.cpp),
//   the warm-started sequential-impulse solve
//   (src/dynamics/free_body_solver.cpp), the position update.
// Every float operation is the host World's (csrc/host/rigid_contacts.cpp,
// csrc/host/novaphy_host.cpp) in the same order, so a served scene's bodies
// follow FluidWorld::step bit for bit.  The translation unit that includes
// this header is compiled with -fmad=false and IEEE division and square root,
// and std::max / std::min are written out as the ternaries they are, which
// keeps their choice between signed zeros and NaN.
#pragma once

#include "novaphy_pbf.h"
#include "rigid_step.hpp"

namespace pbf {
namespace rw {

constexpr int kMaxShapes = 16;
constexpr int kMaxContacts = kMaxShapes * (kMaxShapes - 1) / 2;  // one per pair

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 mul(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 divs(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ V3 normalized(V3 a) {
    const float n2 = dot(a, a);
    if (n2 > 0.0f) {
        const float n = sqrtf(n2);
        return {a.x / n, a.y / n, a.z / n};
    }
    return a;
}
__device__ __forceinline__ float fmax_std(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float fmin_std(float a, float b) { return (b < a) ? b : a; }

struct Q4 {
    float w, x, y, z;
};
// v' = v + w t + q.vec x t with t = 2 (q.vec x v)
__device__ __forceinline__ V3 rotate(const Q4& q, V3 v) {
    const V3 qv{q.x, q.y, q.z};
    V3 t = cross(qv, v);
    t = add(t, t);
    return add(add(v, V3{q.w * t.x, q.w * t.y, q.w * t.z}), cross(qv, t));
}

struct M3 {
    float m[9];
};
__device__ __forceinline__ M3 rotation_matrix(const Q4& q) {
    const float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z, xy = q.x * q.y, xz = q.x * q.z,
                yz = q.y * q.z;
    const float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    return M3{{1.0f - 2.0f * (yy + zz), 2.0f * (xy - wz), 2.0f * (xz + wy), 2.0f * (xy + wz),
               1.0f - 2.0f * (xx + zz), 2.0f * (yz - wx), 2.0f * (xz - wy), 2.0f * (yz + wx),
               1.0f - 2.0f * (xx + yy)}};
}
__device__ __forceinline__ M3 mat_mul(const M3& a, const M3& b) {
    M3 c;
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 3; ++k)
            c.m[3 * r + k] =
                a.m[3 * r] * b.m[k] + (a.m[3 * r + 1] * b.m[3 + k] + a.m[3 * r + 2] * b.m[6 + k]);
    return c;
}
__device__ __forceinline__ M3 transposed(const M3& a) {
    return M3{{a.m[0], a.m[3], a.m[6], a.m[1], a.m[4], a.m[7], a.m[2], a.m[5], a.m[8]}};
}
__device__ __forceinline__ V3 mat_vec(const M3& m, V3 v) {
    return {m.m[0] * v.x + (m.m[1] * v.y + m.m[2] * v.z), m.m[3] * v.x + (m.m[4] * v.y + m.m[5] * v.z),
            m.m[6] * v.x + (m.m[7] * v.y + m.m[8] * v.z)};
}

struct Contact {
    V3 position, normal;
    float penetration;
    int body_a, body_b;
    float friction, restitution;
    float acc_n, acc_t1, acc_t2;
};

struct Row {
    V3 r_a, r_b, t1, t2;
    float k_n, k_t1, k_t2, bias;
    M3 inv_i_a, inv_i_b;
};

// Shared memory of the one-thread pipeline.
struct World {
    V3 pos[kMaxShapes];  // shape centres (spheres)
    V3 lo[kMaxShapes], hi[kMaxShapes];
    int fixed[kMaxShapes];
    Contact c[kMaxContacts];
    Row w[kMaxContacts];
};

__device__ __forceinline__ V3 body_pos(const pbf_rigid_body& b) { return {b.pos[0], b.pos[1], b.pos[2]}; }
__device__ __forceinline__ Q4 body_quat(const pbf_rigid_body& b) {
    return {b.quat[0], b.quat[1], b.quat[2], b.quat[3]};
}
__device__ __forceinline__ V3 lin_of(const pbf_rigid_body& b) {
    return {b.lin_vel[0], b.lin_vel[1], b.lin_vel[2]};
}
__device__ __forceinline__ V3 ang_of(const pbf_rigid_body& b) {
    return {b.ang_vel[0], b.ang_vel[1], b.ang_vel[2]};
}
__device__ __forceinline__ void set_lin(pbf_rigid_body& b, V3 v) {
    b.lin_vel[0] = v.x;
    b.lin_vel[1] = v.y;
    b.lin_vel[2] = v.z;
}
__device__ __forceinline__ void set_ang(pbf_rigid_body& b, V3 v) {
    b.ang_vel[0] = v.x;
    b.ang_vel[1] = v.y;
    b.ang_vel[2] = v.z;
}

// One step of the scene's bodies (after the coupling added force3/torque3
// for the first nforce bodies).  Returns 0, or 1 when a shape is neither a
// sphere nor a plane or names a missing body (the bodies are left as they
// were).
__device__ inline int world_step(World& W, pbf_rigid_body* bodies, int nbodies,
                                 const pbf_rigid_shape* shapes, int nshapes,
                                 const pbf_contact_settings& set, const float* force3,
                                 const float* torque3, int nforce, const float g[3], float dt) {
    if (nshapes > kMaxShapes) return 1;
    for (int k = 0; k < nshapes; ++k) {
        const pbf_rigid_shape& s = shapes[k];
        if (s.type == PBF_SHAPE_SPHERE) {
            if (s.body >= nbodies) return 1;
        } else if (s.type != PBF_SHAPE_PLANE) {
            return 1;
        }
    }
    auto moves = [&](int b) { return b >= 0 && bodies[b].inv_mass > 0.0f; };
    // 1. velocities (world.cpp integrate_velocity)
    for (int i = 0; i < nbodies; ++i) {
        pbf_rigid_body& r = bodies[i];
        if (!(r.inv_mass > 0.0f)) continue;
        float f[3] = {0.0f, 0.0f, 0.0f}, t[3] = {0.0f, 0.0f, 0.0f};
        if (i < nforce)
            for (int d = 0; d < 3; ++d) {
                f[d] = force3[3 * i + d];
                t[d] = torque3[3 * i + d];
            }
        pbf_rigid::integrate_velocity(r.lin_vel, r.ang_vel, g, f, r.inv_mass, r.inv_inertia, t, dt);
    }
    // 2. shape boxes: a sphere's centre +- radius, a plane's +-1e6
    //    (CollisionShape::compute_aabb); fixed: world-owned or on a static body
    for (int k = 0; k < nshapes; ++k) {
        const pbf_rigid_shape& s = shapes[k];
        if (s.type == PBF_SHAPE_SPHERE && s.body >= 0) {
            const pbf_rigid_body& b = bodies[s.body];
            const V3 c = add(body_pos(b), rotate(body_quat(b), V3{s.local_pos[0], s.local_pos[1],
                                                                  s.local_pos[2]}));
            W.pos[k] = c;
            W.lo[k] = sub(c, V3{s.radius, s.radius, s.radius});
            W.hi[k] = add(c, V3{s.radius, s.radius, s.radius});
            W.fixed[k] = !(b.inv_mass > 0.0f);
        } else if (s.type == PBF_SHAPE_SPHERE) {
            // A world-owned sphere: its local centre is its world centre.
            const V3 c{s.local_pos[0], s.local_pos[1], s.local_pos[2]};
            W.pos[k] = c;
            W.lo[k] = sub(c, V3{s.radius, s.radius, s.radius});
            W.hi[k] = add(c, V3{s.radius, s.radius, s.radius});
            W.fixed[k] = 1;
        } else {
            W.pos[k] = V3{0.0f, 0.0f, 0.0f};
            W.lo[k] = V3{-1e6f, -1e6f, -1e6f};
            W.hi[k] = V3{1e6f, 1e6f, 1e6f};
            W.fixed[k] = 1;
        }
    }
    // 3. broad phase + narrow phase, pairs in (lower, higher) order
    int nc = 0;
    for (int a = 0; a < nshapes; ++a)
        for (int b = a + 1; b < nshapes; ++b) {
            if (W.fixed[a] && W.fixed[b]) continue;
            const bool ov = (W.lo[a].x <= W.hi[b].x && W.hi[a].x >= W.lo[b].x) &&
                            (W.lo[a].y <= W.hi[b].y && W.hi[a].y >= W.lo[b].y) &&
                            (W.lo[a].z <= W.hi[b].z && W.hi[a].z >= W.lo[b].z);
            if (!ov) continue;
            const pbf_rigid_shape& sa = shapes[a];
            const pbf_rigid_shape& sb = shapes[b];
            Contact c;
            bool hit = false;
            if (sa.type == PBF_SHAPE_SPHERE && sb.type == PBF_SHAPE_SPHERE) {
                const V3 ca = W.pos[a], cb = W.pos[b];
                const V3 diff = sub(cb, ca);
                const float d2 = dot(diff, diff);
                const float rsum = sa.radius + sb.radius;
                if (!(d2 > rsum * rsum)) {
                    const float dist = sqrtf(d2);
                    const V3 n = dist < 1e-6f ? V3{0.0f, 1.0f, 0.0f} : divs(diff, dist);
                    const float pen = rsum - dist;
                    c.normal = n;
                    c.penetration = pen;
                    c.position = add(ca, mul(n, sa.radius - pen * 0.5f));
                    c.body_a = sa.body;
                    c.body_b = sb.body;
                    hit = true;
                }
            } else if (sa.type != sb.type) {
                // sphere-plane, the plane first in the contact
                const pbf_rigid_shape& sp = sa.type == PBF_SHAPE_SPHERE ? sa : sb;
                const pbf_rigid_shape& pl = sa.type == PBF_SHAPE_SPHERE ? sb : sa;
                const V3 cs = W.pos[sa.type == PBF_SHAPE_SPHERE ? a : b];
                const V3 pn{pl.normal[0], pl.normal[1], pl.normal[2]};
                const float dist = dot(pn, cs) - pl.offset;
                if (!(dist > sp.radius)) {
                    c.normal = pn;
                    c.penetration = sp.radius - dist;
                    c.position = sub(cs, mul(pn, dist));
                    c.body_a = pl.body;
                    c.body_b = sp.body;
                    hit = true;
                }
            }
            if (!hit) continue;
            // World's pipeline sets the pair's material (world.cpp)
            c.friction = sqrtf(sa.friction * sb.friction);
            c.restitution = fmax_std(sa.restitution, sb.restitution);
            c.acc_n = c.acc_t1 = c.acc_t2 = 0.0f;
            W.c[nc++] = c;
        }
    // 4. contact solve (free_body_solver.cpp)
    if (nc > 0) {
        for (int i = 0; i < nc; ++i) {
            Contact& c = W.c[i];
            Row& w = W.w[i];
            w.r_a = c.body_a >= 0 ? sub(c.position, body_pos(bodies[c.body_a])) : V3{0.0f, 0.0f, 0.0f};
            w.r_b = c.body_b >= 0 ? sub(c.position, body_pos(bodies[c.body_b])) : V3{0.0f, 0.0f, 0.0f};
            const float ima = c.body_a >= 0 ? bodies[c.body_a].inv_mass : 0.0f;
            const float imb = c.body_b >= 0 ? bodies[c.body_b].inv_mass : 0.0f;
            auto world_inv = [&](int b) {
                M3 z;
                for (int d = 0; d < 9; ++d) z.m[d] = 0.0f;
                if (!moves(b)) return z;
                const M3 r = rotation_matrix(body_quat(bodies[b]));
                M3 ii;
                for (int d = 0; d < 9; ++d) ii.m[d] = bodies[b].inv_inertia[d];
                return mat_mul(mat_mul(r, ii), transposed(r));
            };
            w.inv_i_a = world_inv(c.body_a);
            w.inv_i_b = world_inv(c.body_b);
            auto eff_mass = [&](V3 u) {
                const V3 ra = cross(w.r_a, u), rb = cross(w.r_b, u);
                float k = ima + imb + dot(ra, mat_vec(w.inv_i_a, ra)) + dot(rb, mat_vec(w.inv_i_b, rb));
                if (k > 0) k = 1.0f / k;
                return k;
            };
            w.k_n = eff_mass(c.normal);
            w.t1 = normalized(fabsf(c.normal.x) < 0.9f ? cross(c.normal, V3{1.0f, 0.0f, 0.0f})
                                                       : cross(c.normal, V3{0.0f, 1.0f, 0.0f}));
            w.t2 = cross(c.normal, w.t1);
            w.k_t1 = eff_mass(w.t1);
            w.k_t2 = eff_mass(w.t2);
            const float depth = fmax_std(0.0f, c.penetration - set.slop);
            w.bias = set.baumgarte * depth / dt;
            const V3 va = c.body_a >= 0 ? add(lin_of(bodies[c.body_a]), cross(ang_of(bodies[c.body_a]), w.r_a))
                                        : V3{0.0f, 0.0f, 0.0f};
            const V3 vb = c.body_b >= 0 ? add(lin_of(bodies[c.body_b]), cross(ang_of(bodies[c.body_b]), w.r_b))
                                        : V3{0.0f, 0.0f, 0.0f};
            const float vn = dot(c.normal, sub(vb, va));
            if (vn < -1.0f) w.bias += c.restitution * vn;
            if (!set.warm_starting) c.acc_n = c.acc_t1 = c.acc_t2 = 0.0f;
        }
        if (set.warm_starting) {
            for (int i = 0; i < nc; ++i) {
                const Contact& c = W.c[i];
                const Row& w = W.w[i];
                if (w.k_n == 0.0f) continue;
                const V3 p = add(add(mul(c.normal, c.acc_n), mul(w.t1, c.acc_t1)), mul(w.t2, c.acc_t2));
                if (moves(c.body_a)) {
                    pbf_rigid_body& b = bodies[c.body_a];
                    set_lin(b, sub(lin_of(b), mul(p, b.inv_mass)));
                    set_ang(b, sub(ang_of(b), mat_vec(w.inv_i_a, cross(w.r_a, p))));
                }
                if (moves(c.body_b)) {
                    pbf_rigid_body& b = bodies[c.body_b];
                    set_lin(b, add(lin_of(b), mul(p, b.inv_mass)));
                    set_ang(b, add(ang_of(b), mat_vec(w.inv_i_b, cross(w.r_b, p))));
                }
            }
        }
        for (int it = 0; it < set.velocity_iterations; ++it) {
            for (int i = 0; i < nc; ++i) {
                Contact& c = W.c[i];
                const Row& w = W.w[i];
                if (w.k_n == 0.0f) continue;
                const float ima = c.body_a >= 0 ? bodies[c.body_a].inv_mass : 0.0f;
                const float imb = c.body_b >= 0 ? bodies[c.body_b].inv_mass : 0.0f;
                const bool ma = moves(c.body_a), mb = moves(c.body_b);
                auto push = [&](V3 p) {
                    if (ma) {
                        pbf_rigid_body& b = bodies[c.body_a];
                        set_lin(b, sub(lin_of(b), mul(p, ima)));
                        set_ang(b, sub(ang_of(b), mat_vec(w.inv_i_a, cross(w.r_a, p))));
                    }
                    if (mb) {
                        pbf_rigid_body& b = bodies[c.body_b];
                        set_lin(b, add(lin_of(b), mul(p, imb)));
                        set_ang(b, add(ang_of(b), mat_vec(w.inv_i_b, cross(w.r_b, p))));
                    }
                };
                auto rel_vel = [&]() {
                    const V3 va = c.body_a >= 0
                                      ? add(lin_of(bodies[c.body_a]), cross(ang_of(bodies[c.body_a]), w.r_a))
                                      : V3{0.0f, 0.0f, 0.0f};
                    const V3 vb = c.body_b >= 0
                                      ? add(lin_of(bodies[c.body_b]), cross(ang_of(bodies[c.body_b]), w.r_b))
                                      : V3{0.0f, 0.0f, 0.0f};
                    return sub(vb, va);
                };
                float dn = w.k_n * (-dot(rel_vel(), c.normal) + w.bias);
                const float old_n = c.acc_n;
                c.acc_n = fmax_std(0.0f, old_n + dn);
                dn = c.acc_n - old_n;
                push(mul(c.normal, dn));
                const float cap = c.friction * c.acc_n;
                float d1 = w.k_t1 * -dot(rel_vel(), w.t1);
                const float old_1 = c.acc_t1;
                c.acc_t1 = fmax_std(-cap, fmin_std(cap, old_1 + d1));
                d1 = c.acc_t1 - old_1;
                push(mul(w.t1, d1));
                float d2 = w.k_t2 * -dot(rel_vel(), w.t2);
                const float old_2 = c.acc_t2;
                c.acc_t2 = fmax_std(-cap, fmin_std(cap, old_2 + d2));
                d2 = c.acc_t2 - old_2;
                push(mul(w.t2, d2));
            }
        }
    }
    // 5. positions (world.cpp integrate_position)
    for (int i = 0; i < nbodies; ++i) {
        pbf_rigid_body& r = bodies[i];
        if (!(r.inv_mass > 0.0f)) continue;
        pbf_rigid::integrate_position(r.pos, r.quat, r.lin_vel, r.ang_vel, dt);
    }
    return 0;
}

}  // namespace rw
}  // namespace pbf
