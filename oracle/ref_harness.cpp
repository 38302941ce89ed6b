// C-ABI harness around the reference's own PBF sources (test infrastructure
// only: the tests use it to pin the oracle restatement; the product never
// links it).  Built by oracle/build_oracle.py into oracle/_ref/ from the
// reference's unmodified files
//   src/fluid/pbf_solver.cpp, src/fluid/neighbor_search.cpp,
//   src/fluid/particle_state.cpp, src/fluid/boundary.cpp,
//   src/fluid/fluid_world.cpp, src/sim/performance_monitor.cpp, and the rigid
//   pipeline FluidWorld inherits (src/sim/world.cpp, state.cpp, src/core/
//   body.cpp, shape.cpp, model_builder.cpp, joint.cpp, src/collision/*.cpp,
//   src/dynamics/free_body_solver.cpp, integrator.cpp, src/math/*.cpp)
// against the Eigen-API subset in oracle/eigen_shim (Eigen3 is absent here).
#include <cstring>
#include <vector>

#include "novaphy/collision/broadphase.h"
#include "novaphy/collision/narrowphase.h"
#include "novaphy/core/model_builder.h"
#include "novaphy/fluid/boundary.h"
#include "novaphy/fluid/fluid_world.h"
#include "novaphy/fluid/neighbor_search.h"
#include "novaphy/fluid/particle_state.h"
#include "novaphy/fluid/pbf_solver.h"
#include "novaphy/fluid/sph_kernel.h"

using namespace novaphy;

extern "C" {

// Same field order as the oracle's orc_settings and the product's pbf_settings.
struct ref_settings {
    float rest_density;
    float kernel_radius;
    float particle_radius;
    int solver_iterations;
    float epsilon;
    float xsph_viscosity;
    float vorticity_epsilon;
    float corr_delta_q;
    float corr_k;
    int corr_n;
    int use_domain_bounds;
    float domain_lower[3];
    float domain_upper[3];
};

static PBFSettings to_settings(const ref_settings* s) {
    PBFSettings p;
    p.rest_density = s->rest_density;
    p.kernel_radius = s->kernel_radius;
    p.particle_radius = s->particle_radius;
    p.solver_iterations = s->solver_iterations;
    p.epsilon = s->epsilon;
    p.xsph_viscosity = s->xsph_viscosity;
    p.vorticity_epsilon = s->vorticity_epsilon;
    p.corr_delta_q = s->corr_delta_q;
    p.corr_k = s->corr_k;
    p.corr_n = s->corr_n;
    p.use_domain_bounds = s->use_domain_bounds != 0;
    p.domain_lower = Vec3f(s->domain_lower[0], s->domain_lower[1], s->domain_lower[2]);
    p.domain_upper = Vec3f(s->domain_upper[0], s->domain_upper[1], s->domain_upper[2]);
    return p;
}

void ref_default_settings(ref_settings* out) {
    PBFSettings d;
    out->rest_density = d.rest_density;
    out->kernel_radius = d.kernel_radius;
    out->particle_radius = d.particle_radius;
    out->solver_iterations = d.solver_iterations;
    out->epsilon = d.epsilon;
    out->xsph_viscosity = d.xsph_viscosity;
    out->vorticity_epsilon = d.vorticity_epsilon;
    out->corr_delta_q = d.corr_delta_q;
    out->corr_k = d.corr_k;
    out->corr_n = d.corr_n;
    out->use_domain_bounds = d.use_domain_bounds ? 1 : 0;
    for (int c = 0; c < 3; ++c) {
        out->domain_lower[c] = d.domain_lower[c];
        out->domain_upper[c] = d.domain_upper[c];
    }
}

// Runs `nsteps` reference PBF steps on host arrays (x, v: n*3; rho, lam: n),
// in place.  rho/lam are loaded into the state first because the reference
// reads the previous densities when solver_iterations == 0.
int ref_pbf_steps(const ref_settings* s, int n, float* x, float* v, float* rho, float* lam,
                  float dt, const float* g, float mass, int nsteps) {
    PBFSolver solver(to_settings(s));
    ParticleState st;
    std::vector<Vec3f> pos(n);
    for (int i = 0; i < n; ++i) pos[i] = Vec3f(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
    st.init(pos);
    for (int i = 0; i < n; ++i) {
        st.velocities[i] = Vec3f(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        st.densities[i] = rho[i];
        st.lambdas[i] = lam[i];
    }
    const Vec3f gv(g[0], g[1], g[2]);
    for (int k = 0; k < nsteps; ++k) solver.step(st, dt, gv, mass);
    for (int i = 0; i < n; ++i) {
        for (int c = 0; c < 3; ++c) {
            x[3 * i + c] = st.positions[i][c];
            v[3 * i + c] = st.velocities[i][c];
        }
        rho[i] = st.densities[i];
        lam[i] = st.lambdas[i];
    }
    return 0;
}

// SpatialHashGrid: build over `n` points, query the candidate list of point q.
// Writes up to `cap` indices, returns the full count.
int ref_grid_query(const float* pts, int n, float cell, const float* q, float radius, int* out,
                   int cap) {
    std::vector<Vec3f> p(n);
    for (int i = 0; i < n; ++i) p[i] = Vec3f(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
    SpatialHashGrid grid(cell);
    grid.build(p);
    std::vector<int> res;
    grid.query_neighbors(Vec3f(q[0], q[1], q[2]), radius, res);
    const int m = static_cast<int>(res.size());
    for (int i = 0; i < m && i < cap; ++i) out[i] = res[i];
    return m;
}

// query_all_pairs: writes pairs as (i, j) int pairs, returns the pair count.
int ref_query_all_pairs(const float* pts, int n, float cell, float radius, int* out, int cap) {
    std::vector<Vec3f> p(n);
    for (int i = 0; i < n; ++i) p[i] = Vec3f(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
    SpatialHashGrid grid(cell);
    grid.build(p);
    auto pairs = grid.query_all_pairs(p, radius);
    const int m = static_cast<int>(pairs.size());
    for (int k = 0; k < m && k < cap; ++k) {
        out[2 * k] = pairs[k].first;
        out[2 * k + 1] = pairs[k].second;
    }
    return m;
}

// generate_fluid_block: writes up to `cap` positions, returns the count.
int ref_generate_block(const float* lower, const float* upper, float spacing, float* out,
                       int cap) {
    FluidBlockDef d;
    d.lower = Vec3f(lower[0], lower[1], lower[2]);
    d.upper = Vec3f(upper[0], upper[1], upper[2]);
    d.particle_spacing = spacing;
    auto pos = generate_fluid_block(d);
    const int m = static_cast<int>(pos.size());
    for (int i = 0; i < m && i < cap; ++i)
        for (int c = 0; c < 3; ++c) out[3 * i + c] = pos[i][c];
    return m;
}

float ref_poly6(float r_sq, float h) { return SPHKernels::poly6(r_sq, h); }
float ref_spiky(float r, float h) { return SPHKernels::spiky(r, h); }
float ref_cubic_spline(float r, float h) { return SPHKernels::cubic_spline(r, h); }
void ref_spiky_grad(const float* r, float h, float* out) {
    Vec3f g = SPHKernels::spiky_grad(Vec3f(r[0], r[1], r[2]), h);
    for (int c = 0; c < 3; ++c) out[c] = g[c];
}

// Samplers (boundary.cpp:15-126) on a shape built from its fields; they write
// up to cap body-frame positions and return the count.
static int copy_samples(const std::vector<BoundaryParticle>& bp, float* out3, int cap) {
    const int m = (int)bp.size();
    if (out3)
        for (int i = 0; i < m && i < cap; ++i)
            for (int d = 0; d < 3; ++d) out3[3 * i + d] = bp[(size_t)i].local_position(d);
    return m;
}

static Transform local_tf(const float* lt_pos, const float* lt_quat) {
    Transform t;
    t.position = Vec3f(lt_pos[0], lt_pos[1], lt_pos[2]);
    t.rotation = Quatf(lt_quat[0], lt_quat[1], lt_quat[2], lt_quat[3]);
    return t;
}

int ref_sample_box(const float* half, const float* lt_pos, const float* lt_quat, float spacing,
                   float* out3, int cap) {
    CollisionShape s;
    s.type = ShapeType::Box;
    s.box.half_extents = Vec3f(half[0], half[1], half[2]);
    s.local_transform = local_tf(lt_pos, lt_quat);
    s.body_index = 0;
    return copy_samples(sample_box_boundary(s, spacing), out3, cap);
}

int ref_sample_sphere(float radius, const float* lt_pos, const float* lt_quat, float spacing,
                      float* out3, int cap) {
    CollisionShape s;
    s.type = ShapeType::Sphere;
    s.sphere.radius = radius;
    s.local_transform = local_tf(lt_pos, lt_quat);
    s.body_index = 0;
    return copy_samples(sample_sphere_boundary(s, spacing), out3, cap);
}

int ref_sample_plane(const float* normal, float offset, float spacing, float extent, float* out3,
                     int cap) {
    CollisionShape s;
    s.type = ShapeType::Plane;
    s.plane.normal = Vec3f(normal[0], normal[1], normal[2]);
    s.plane.offset = offset;
    return copy_samples(sample_plane_boundary(s, spacing, extent), out3, cap);
}

// FluidWorld::step (fluid_world.cpp:46-99) over nsteps steps of a world with
// one fluid block and nb bodies: kind[k] 0 = sphere (size[3k] = radius),
// 1 = box (size[3k..3k+2] = half extents), mass[k], pose pos3/quat4 (w, x, y,
// z; normalised), plus, when with_plane, a plane make_plane(plane_normal3,
// plane_offset) with the default friction and restitution.  The world's
// gravity is gravity3 (null: the World default (0, -9.81, 0)).  Writes the
// fluid state (n particles, as ParticleState) and the bodies' poses and
// velocities; returns n, or -1.
int ref_fluid_world_run_ex(const ref_settings* st, const float* lower, const float* upper,
                           float spacing, int nb, const int* kind, const float* size,
                           const float* mass, const float* pos3, const float* quat4,
                           int with_plane, const float* plane_normal3, float plane_offset,
                           float boundary_extent, const float* gravity3, float dt, int nsteps,
                           int cap, float* x3, float* v3, float* rho, float* lam,
                           float* body_pos3, float* body_quat4, float* body_v3, float* body_w3) {
    try {
        ModelBuilder mb;
        if (with_plane)
            mb.add_shape(CollisionShape::make_plane(
                Vec3f(plane_normal3[0], plane_normal3[1], plane_normal3[2]), plane_offset));
        for (int k = 0; k < nb; ++k) {
            // Transform(p, q) normalises q, as the reference's Python API does.
            const Transform t(Vec3f(pos3[3 * k], pos3[3 * k + 1], pos3[3 * k + 2]),
                              Quatf(quat4[4 * k], quat4[4 * k + 1], quat4[4 * k + 2],
                                    quat4[4 * k + 3]));
            if (kind[k] == 0) {
                const int b = mb.add_body(RigidBody::from_sphere(mass[k], size[3 * k]), t);
                mb.add_shape(CollisionShape::make_sphere(size[3 * k], b));
            } else {
                const Vec3f he(size[3 * k], size[3 * k + 1], size[3 * k + 2]);
                const int b = mb.add_body(RigidBody::from_box(mass[k], he), t);
                mb.add_shape(CollisionShape::make_box(he, b));
            }
        }
        FluidBlockDef blk;
        blk.lower = Vec3f(lower[0], lower[1], lower[2]);
        blk.upper = Vec3f(upper[0], upper[1], upper[2]);
        blk.particle_spacing = spacing;
        FluidWorld fw(mb.build(), {blk}, SolverSettings{}, to_settings(st), boundary_extent);
        if (gravity3) fw.set_gravity(Vec3f(gravity3[0], gravity3[1], gravity3[2]));
        for (int s = 0; s < nsteps; ++s) fw.step(dt);
        const ParticleState& ps = fw.fluid_state();
        const int n = ps.num_particles();
        if (n > cap) return -1;
        for (int i = 0; i < n; ++i) {
            for (int d = 0; d < 3; ++d) {
                x3[3 * i + d] = ps.positions[(size_t)i](d);
                v3[3 * i + d] = ps.velocities[(size_t)i](d);
            }
            rho[i] = ps.densities[(size_t)i];
            lam[i] = ps.lambdas[(size_t)i];
        }
        const SimState& ss = fw.state();
        for (int k = 0; k < nb; ++k) {
            const Transform& t = ss.transforms[(size_t)k];
            for (int d = 0; d < 3; ++d) {
                body_pos3[3 * k + d] = t.position(d);
                body_v3[3 * k + d] = ss.linear_velocities[(size_t)k](d);
                body_w3[3 * k + d] = ss.angular_velocities[(size_t)k](d);
            }
            body_quat4[4 * k] = t.rotation.w();
            body_quat4[4 * k + 1] = t.rotation.x();
            body_quat4[4 * k + 2] = t.rotation.y();
            body_quat4[4 * k + 3] = t.rotation.z();
        }
        return n;
    } catch (...) {
        return -1;
    }
}

// ref_fluid_world_run_ex with the ground plane of add_ground_plane(plane_y)
// (normal +y, model_builder.cpp:42-46) and the World's default gravity.
int ref_fluid_world_run(const ref_settings* st, const float* lower, const float* upper,
                        float spacing, int nb, const int* kind, const float* size,
                        const float* mass, const float* pos3, const float* quat4, int with_plane,
                        float plane_y, float boundary_extent, float dt, int nsteps, int cap,
                        float* x3, float* v3, float* rho, float* lam, float* body_pos3,
                        float* body_quat4, float* body_v3, float* body_w3) {
    const float up[3] = {0.0f, 1.0f, 0.0f};
    return ref_fluid_world_run_ex(st, lower, upper, spacing, nb, kind, size, mass, pos3, quat4,
                                  with_plane, up, plane_y, boundary_extent, nullptr, dt, nsteps,
                                  cap, x3, v3, rho, lam, body_pos3, body_quat4, body_v3, body_w3);
}

// World::step (world.cpp) over nsteps steps of nb free bodies (kind, size,
// mass and pose as ref_fluid_world_run) starting from linear and angular
// velocities lin3/ang3, with optional constant forces/torques applied before
// every step (force3/torque3, may be null).  No ground plane.  Writes poses and
// velocities.  Returns 0, or -1.
int ref_world_run(int nb, const int* kind, const float* size, const float* mass,
                  const float* pos3, const float* quat4, const float* lin3, const float* ang3,
                  const float* force3, const float* torque3, float dt, int nsteps,
                  float* body_pos3, float* body_quat4, float* body_v3, float* body_w3) {
    try {
        ModelBuilder mb;
        for (int k = 0; k < nb; ++k) {
            // Transform(p, q) normalises q, as the reference's Python API does.
            const Transform t(Vec3f(pos3[3 * k], pos3[3 * k + 1], pos3[3 * k + 2]),
                              Quatf(quat4[4 * k], quat4[4 * k + 1], quat4[4 * k + 2],
                                    quat4[4 * k + 3]));
            if (kind[k] == 0) {
                const int b = mb.add_body(RigidBody::from_sphere(mass[k], size[3 * k]), t);
                mb.add_shape(CollisionShape::make_sphere(size[3 * k], b));
            } else {
                const Vec3f he(size[3 * k], size[3 * k + 1], size[3 * k + 2]);
                const int b = mb.add_body(RigidBody::from_box(mass[k], he), t);
                mb.add_shape(CollisionShape::make_box(he, b));
            }
        }
        World w(mb.build(), SolverSettings{});
        for (int k = 0; k < nb; ++k) {
            w.state().set_linear_velocity(k, Vec3f(lin3[3 * k], lin3[3 * k + 1], lin3[3 * k + 2]));
            w.state().set_angular_velocity(k, Vec3f(ang3[3 * k], ang3[3 * k + 1], ang3[3 * k + 2]));
        }
        for (int s = 0; s < nsteps; ++s) {
            for (int k = 0; k < nb; ++k) {
                if (force3) w.apply_force(k, Vec3f(force3[3 * k], force3[3 * k + 1], force3[3 * k + 2]));
                if (torque3)
                    w.apply_torque(k, Vec3f(torque3[3 * k], torque3[3 * k + 1], torque3[3 * k + 2]));
            }
            w.step(dt);
        }
        const SimState& ss = w.state();
        for (int k = 0; k < nb; ++k) {
            const Transform& t = ss.transforms[(size_t)k];
            for (int d = 0; d < 3; ++d) {
                body_pos3[3 * k + d] = t.position(d);
                body_v3[3 * k + d] = ss.linear_velocities[(size_t)k](d);
                body_w3[3 * k + d] = ss.angular_velocities[(size_t)k](d);
            }
            body_quat4[4 * k] = t.rotation.w();
            body_quat4[4 * k + 1] = t.rotation.x();
            body_quat4[4 * k + 2] = t.rotation.y();
            body_quat4[4 * k + 3] = t.rotation.z();
        }
        return 0;
    } catch (...) {
        return -1;
    }
}

// Akinci volumes of boundary particles at world positions
// (compute_boundary_volumes, boundary.cpp:152-176).  1 if it throws.
int ref_boundary_volumes(int nb, const float* world3, float h, float* psi) {
    std::vector<BoundaryParticle> bp((size_t)nb);
    std::vector<Vec3f> w((size_t)nb);
    for (int i = 0; i < nb; ++i) w[(size_t)i] = Vec3f(world3[3 * i], world3[3 * i + 1], world3[3 * i + 2]);
    try {
        compute_boundary_volumes(bp, w, h);
    } catch (...) {
        return 1;
    }
    for (int i = 0; i < nb; ++i) psi[i] = bp[(size_t)i].volume;
    return 0;
}

// World positions of boundary particles under body poses (w, x, y, z
// quaternions, taken as given) (boundary_world_positions, boundary.cpp:178-192).
void ref_boundary_world_positions(int nb, const float* local3, const int* body, int nbodies,
                                  const float* pos3, const float* quat4, float* out3) {
    std::vector<BoundaryParticle> bp((size_t)nb);
    for (int i = 0; i < nb; ++i) {
        bp[(size_t)i].local_position = Vec3f(local3[3 * i], local3[3 * i + 1], local3[3 * i + 2]);
        bp[(size_t)i].body_index = body[i];
    }
    std::vector<Transform> tr((size_t)nbodies);
    for (int k = 0; k < nbodies; ++k) {
        tr[(size_t)k].position = Vec3f(pos3[3 * k], pos3[3 * k + 1], pos3[3 * k + 2]);
        tr[(size_t)k].rotation = Quatf(quat4[4 * k], quat4[4 * k + 1], quat4[4 * k + 2], quat4[4 * k + 3]);
    }
    const std::vector<Vec3f> w = boundary_world_positions(bp, tr);
    for (int i = 0; i < nb; ++i)
        for (int d = 0; d < 3; ++d) out3[3 * i + d] = w[(size_t)i](d);
}

// ---- rigid contact pipeline ----
// A shape is 19 floats: type (0 box, 1 sphere, 2 plane), body index,
// half extents (3), radius, plane normal (3), plane offset, local position
// (3), local rotation (w, x, y, z), friction, restitution.  A contact is 11
// floats: position (3), normal (3), penetration, body_a, body_b, friction,
// restitution.
static CollisionShape shape_from(const float* f) {
    CollisionShape s;
    s.type = f[0] == 0.0f ? ShapeType::Box : (f[0] == 1.0f ? ShapeType::Sphere : ShapeType::Plane);
    s.body_index = (int)f[1];
    s.box.half_extents = Vec3f(f[2], f[3], f[4]);
    s.sphere.radius = f[5];
    s.plane.normal = Vec3f(f[6], f[7], f[8]);
    s.plane.offset = f[9];
    s.local_transform = Transform(Vec3f(f[10], f[11], f[12]), Quatf(f[13], f[14], f[15], f[16]));
    s.friction = f[17];
    s.restitution = f[18];
    return s;
}

static void contact_to(const ContactPoint& c, float* o) {
    for (int d = 0; d < 3; ++d) {
        o[d] = c.position(d);
        o[3 + d] = c.normal(d);
    }
    o[6] = c.penetration;
    o[7] = (float)c.body_a;
    o[8] = (float)c.body_b;
    o[9] = c.friction;
    o[10] = c.restitution;
}

// collide_shapes on two shapes at poses (position 3, rotation w x y z).
// Writes up to cap contacts; returns their count, with hit in *hit.
int ref_collide(const float* sa, const float* pa7, const float* sb, const float* pb7, float* out,
                int cap, int* hit) {
    const Transform ta(Vec3f(pa7[0], pa7[1], pa7[2]), Quatf(pa7[3], pa7[4], pa7[5], pa7[6]));
    const Transform tb(Vec3f(pb7[0], pb7[1], pb7[2]), Quatf(pb7[3], pb7[4], pb7[5], pb7[6]));
    std::vector<ContactPoint> c;
    *hit = collide_shapes(shape_from(sa), ta, shape_from(sb), tb, c) ? 1 : 0;
    const int n = (int)c.size();
    for (int k = 0; k < n && k < cap; ++k) contact_to(c[(size_t)k], out + 11 * k);
    return n;
}

// SweepAndPrune over n boxes (min 3, max 3 each) and a static mask; writes
// up to cap pairs (a, b); returns the pair count.
int ref_sap(int n, const float* boxes6, const int* fixed, int* pairs2, int cap) {
    std::vector<AABB> a((size_t)n);
    std::vector<bool> m((size_t)n);
    for (int i = 0; i < n; ++i) {
        const float* b = boxes6 + 6 * i;
        a[(size_t)i] = AABB(Vec3f(b[0], b[1], b[2]), Vec3f(b[3], b[4], b[5]));
        m[(size_t)i] = fixed[i] != 0;
    }
    SweepAndPrune sap;
    sap.update(a, m);
    const auto& p = sap.get_pairs();
    for (int k = 0; k < (int)p.size() && k < cap; ++k) {
        pairs2[2 * k] = p[(size_t)k].body_a;
        pairs2[2 * k + 1] = p[(size_t)k].body_b;
    }
    return (int)p.size();
}

// A rigid World of nb bodies (17 floats each: mass, inertia row-major (9),
// position (3), rotation (w, x, y, z)) and ns shapes (19 floats each, as
// above), with initial velocities lin3/ang3, solver settings (8 floats:
// velocity_iterations, baumgarte, slop, warm_starting, sleep_enabled,
// sleep_energy_threshold, sleep_time_required, sleep_ema_alpha) and gravity,
// stepped nsteps times.  Writes the final poses and velocities, the contact
// count of every step and the final sleep flags.  Returns 0, or -1.
int ref_rigid_world_run(int nb, const float* bodies17, int ns, const float* shapes19,
                        const float* lin3, const float* ang3, const float* settings8,
                        const float* gravity3, float dt, int nsteps, float* body_pos3,
                        float* body_quat4, float* body_v3, float* body_w3, int* contacts_per_step,
                        int* sleeping) {
    try {
        ModelBuilder mb;
        for (int k = 0; k < nb; ++k) {
            const float* b = bodies17 + 17 * k;
            RigidBody rb;
            rb.mass = b[0];
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) rb.inertia(r, c) = b[1 + 3 * r + c];
            mb.add_body(rb, Transform(Vec3f(b[10], b[11], b[12]), Quatf(b[13], b[14], b[15], b[16])));
        }
        for (int k = 0; k < ns; ++k) mb.add_shape(shape_from(shapes19 + 19 * k));
        SolverSettings st;
        st.velocity_iterations = (int)settings8[0];
        st.baumgarte = settings8[1];
        st.slop = settings8[2];
        st.warm_starting = settings8[3] != 0.0f;
        st.sleep_enabled = settings8[4] != 0.0f;
        st.sleep_energy_threshold = settings8[5];
        st.sleep_time_required = settings8[6];
        st.sleep_ema_alpha = settings8[7];
        World w(mb.build(), st);
        w.set_gravity(Vec3f(gravity3[0], gravity3[1], gravity3[2]));
        for (int k = 0; k < nb; ++k) {
            w.state().set_linear_velocity(k, Vec3f(lin3[3 * k], lin3[3 * k + 1], lin3[3 * k + 2]));
            w.state().set_angular_velocity(k, Vec3f(ang3[3 * k], ang3[3 * k + 1], ang3[3 * k + 2]));
        }
        for (int s = 0; s < nsteps; ++s) {
            w.step(dt);
            contacts_per_step[s] = (int)w.contacts().size();
        }
        const SimState& ss = w.state();
        for (int k = 0; k < nb; ++k) {
            const Transform& t = ss.transforms[(size_t)k];
            for (int d = 0; d < 3; ++d) {
                body_pos3[3 * k + d] = t.position(d);
                body_v3[3 * k + d] = ss.linear_velocities[(size_t)k](d);
                body_w3[3 * k + d] = ss.angular_velocities[(size_t)k](d);
            }
            body_quat4[4 * k] = t.rotation.w();
            body_quat4[4 * k + 1] = t.rotation.x();
            body_quat4[4 * k + 2] = t.rotation.y();
            body_quat4[4 * k + 3] = t.rotation.z();
            sleeping[k] = ss.sleeping[(size_t)k];
        }
        return 0;
    } catch (...) {
        return -1;
    }
}

}  // extern "C"

