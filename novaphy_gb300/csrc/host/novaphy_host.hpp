// Host layer of the GB300 PBF path: NovaPhy's fluid API (the types of
// include/novaphy/fluid/*.h and the parts of sim/core/math they use) on top
// of the C ABI in include/novaphy_pbf.h.  The PBF step, the neighbour search
// and the Akinci coupling run on the device; setup (fluid blocks, boundary
// sampling) and the small rigid-body state stay on the host.
#pragma once

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "novaphy_pbf.h"

namespace novaphy_gb300 {

constexpr float kPi = 3.14159265358979323846f;

// 3-vector with the reference's arithmetic (Eigen::Vector3f): component-wise
// ops, 3-term reductions as e0 + (e1 + e2).
struct Vec3 {
    float x = 0.0f, y = 0.0f, z = 0.0f;
    Vec3() = default;
    Vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    Vec3 operator+(const Vec3& o) const { return {x + o.x, y + o.y, z + o.z}; }
    Vec3 operator-(const Vec3& o) const { return {x - o.x, y - o.y, z - o.z}; }
    Vec3 operator*(float s) const { return {x * s, y * s, z * s}; }
    Vec3 operator/(float s) const { return {x / s, y / s, z / s}; }
    Vec3 operator-() const { return {-x, -y, -z}; }
    Vec3& operator+=(const Vec3& o) {
        x = x + o.x;
        y = y + o.y;
        z = z + o.z;
        return *this;
    }
    Vec3& operator-=(const Vec3& o) {
        x = x - o.x;
        y = y - o.y;
        z = z - o.z;
        return *this;
    }
    float dot(const Vec3& o) const { return x * o.x + (y * o.y + z * o.z); }
    float squaredNorm() const { return dot(*this); }
    float norm() const { return std::sqrt(squaredNorm()); }
    Vec3 cross(const Vec3& o) const {
        return {y * o.z - z * o.y, z * o.x - x * o.z, x * o.y - y * o.x};
    }
    Vec3 normalized() const {
        const float n2 = squaredNorm();
        if (n2 > 0.0f) {
            const float n = std::sqrt(n2);
            return {x / n, y / n, z / n};
        }
        return *this;
    }
};
inline Vec3 operator*(float s, const Vec3& v) { return {s * v.x, s * v.y, s * v.z}; }
static_assert(sizeof(Vec3) == 3 * sizeof(float), "Vec3 must be a packed float[3]");

// Row-major 3x3 matrix; products sum their three terms as t0 + (t1 + t2).
using Mat3 = std::array<float, 9>;

// Unit quaternion (w, x, y, z).
struct Quat {
    float w = 1.0f, x = 0.0f, y = 0.0f, z = 0.0f;
    Vec3 vec() const { return {x, y, z}; }
    Quat conjugate() const { return {w, -x, -y, -z}; }
    // Hamilton product, each component summed left to right.
    Quat operator*(const Quat& o) const {
        return {w * o.w - x * o.x - y * o.y - z * o.z, w * o.x + x * o.w + y * o.z - z * o.y,
                w * o.y + y * o.w + z * o.x - x * o.z, w * o.z + z * o.w + x * o.y - y * o.x};
    }
    // R = I + 2 (w [v]x + [v]x^2), written out per entry.
    Mat3 rotation_matrix() const {
        const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z;
        const float wx = w * x, wy = w * y, wz = w * z;
        return {1.0f - 2.0f * (yy + zz), 2.0f * (xy - wz),        2.0f * (xz + wy),
                2.0f * (xy + wz),        1.0f - 2.0f * (xx + zz), 2.0f * (yz - wx),
                2.0f * (xz - wy),        2.0f * (yz + wx),        1.0f - 2.0f * (xx + yy)};
    }
    // v' = v + w t + q.vec x t with t = 2 (q.vec x v)
    Vec3 rotate(const Vec3& v) const {
        Vec3 t = vec().cross(v);
        t = t + t;
        return (v + w * t) + vec().cross(t);
    }
    Quat normalized() const {
        const float n = std::sqrt((w * w + x * x) + (y * y + z * z));
        if (n > 0.0f) return {w / n, x / n, y / n, z / n};
        return *this;
    }
    static Quat from_axis_angle(const Vec3& axis, float angle) {
        const Vec3 a = axis.normalized();
        const float s = std::sin(angle * 0.5f);
        return Quat{std::cos(angle * 0.5f), s * a.x, s * a.y, s * a.z};
    }
};

// Rigid transform (include/novaphy/math/math_types.h:38-135).
struct Transform {
    Vec3 position;
    Quat rotation;
    Transform() = default;
    Transform(const Vec3& p, const Quat& q) : position(p), rotation(q.normalized()) {}
    // Composition and inverse renormalise the rotation, as the constructor does.
    Transform operator*(const Transform& o) const {
        return Transform(position + rotation.rotate(o.position), rotation * o.rotation);
    }
    Transform inverse() const {
        const Quat r = rotation.conjugate();
        return Transform(r.rotate(Vec3(-position.x, -position.y, -position.z)), r);
    }
    Vec3 transform_point(const Vec3& p) const { return position + rotation.rotate(p); }
    Vec3 transform_vector(const Vec3& v) const { return rotation.rotate(v); }
    Mat3 rotation_matrix() const { return rotation.rotation_matrix(); }
    static Transform identity() { return Transform(); }
    static Transform from_translation(const Vec3& t) { return Transform(t, Quat{}); }
    static Transform from_axis_angle(const Vec3& axis, float angle) {
        return Transform(Vec3{}, Quat::from_axis_angle(axis, angle));
    }
};

// PBFSettings (include/novaphy/fluid/pbf_solver.h:13-38) + this library's
// arithmetic and hash-compatibility switches.
struct PBFSettings {
    float rest_density = 1000.0f;
    float kernel_radius = 0.1f;
    float particle_radius = 0.025f;
    int solver_iterations = 4;
    float epsilon = 100.0f;
    float xsph_viscosity = 0.01f;
    float vorticity_epsilon = 0.0f;
    float corr_delta_q = 0.3f;
    float corr_k = 0.001f;
    int corr_n = 4;
    bool use_domain_bounds = false;
    Vec3 domain_lower{-10.0f, 0.0f, -10.0f};
    Vec3 domain_upper{10.0f, 10.0f, 10.0f};
    bool exact_arithmetic = true;
    bool hash_compat = true;
    bool boundary_two_way = false;  // no counterpart in the reference (pbf_settings)
    float boundary_friction = 0.0f;  // two-way only; no counterpart in the reference
    float particle_mass(float spacing) const { return rest_density * spacing * spacing * spacing; }
    ::pbf_settings to_c() const;
};

// SPH kernels on the host (include/novaphy/fluid/sph_kernel.h:16-81).
struct SPHKernels {
    static float poly6(float r_sq, float h);
    static Vec3 spiky_grad(const Vec3& r, float h);
    static float spiky(float r_len, float h);
    static float cubic_spline(float r_len, float h);
};

struct FluidBlockDef {
    Vec3 lower, upper;
    float particle_spacing = 0.02f;
    float rest_density = 1000.0f;
    Vec3 initial_velocity;
};

std::vector<Vec3> generate_fluid_block(const FluidBlockDef& def);

struct ParticleState {
    std::vector<Vec3> positions, velocities;
    std::vector<float> densities, lambdas;
    void init(const std::vector<Vec3>& initial_positions, const Vec3& initial_velocity = Vec3{});
    void clear();
    int num_particles() const { return (int)positions.size(); }
};

// Host spatial hash grid with the reference's keys and bucket order
// (src/fluid/neighbor_search.cpp); used by callers of the API, not by the step.
class SpatialHashGrid {
public:
    explicit SpatialHashGrid(float cell_size = 0.1f) : cell_size_(cell_size) {}
    void build(const std::vector<Vec3>& positions);
    void clear() { cells_.clear(); }
    std::vector<int> query_neighbors(const Vec3& point, float radius) const;
    std::vector<std::pair<int, int>> query_all_pairs(const std::vector<Vec3>& positions,
                                                     float radius) const;
    float cell_size() const { return cell_size_; }
    void set_cell_size(float s) { cell_size_ = s; }
    static uint64_t hash_cell(int cx, int cy, int cz);

private:
    void world_to_cell(const Vec3& p, int& cx, int& cy, int& cz) const;
    float cell_size_;
    std::unordered_map<uint64_t, std::vector<int>> cells_;
};

// ---- rigid-body model (host; the scene description FluidWorld needs) ----

enum class ShapeType { Box, Sphere, Plane };

// Axis-aligned box (include/novaphy/core/aabb.h); the default is empty
// (min = +FLT_MAX, max = -FLT_MAX) so that expand() starts from nothing.
struct AABB {
    Vec3 min{3.402823466e+38f, 3.402823466e+38f, 3.402823466e+38f};
    Vec3 max{-3.402823466e+38f, -3.402823466e+38f, -3.402823466e+38f};
    AABB() = default;
    AABB(const Vec3& lo, const Vec3& hi) : min(lo), max(hi) {}
    bool overlaps(const AABB& o) const {
        return (min.x <= o.max.x && max.x >= o.min.x) && (min.y <= o.max.y && max.y >= o.min.y) &&
               (min.z <= o.max.z && max.z >= o.min.z);
    }
    void expand(const Vec3& p);
    Vec3 center() const { return 0.5f * (min + max); }
    Vec3 half_extents() const { return 0.5f * (max - min); }
    float surface_area() const {
        const Vec3 d = max - min;
        return 2.0f * (d.x * d.y + d.y * d.z + d.z * d.x);
    }
    bool is_valid() const { return min.x <= max.x && min.y <= max.y && min.z <= max.z; }
    static AABB from_sphere(const Vec3& c, float r) {
        return AABB(c - Vec3(r, r, r), c + Vec3(r, r, r));
    }
};

struct CollisionShape {
    ShapeType type = ShapeType::Box;
    int body_index = -1;
    Transform local_transform;
    Vec3 half_extents{0.5f, 0.5f, 0.5f};
    float radius = 0.5f;
    Vec3 normal{0.0f, 1.0f, 0.0f};
    float offset = 0.0f;
    float friction = 0.5f;
    float restitution = 0.3f;
    static CollisionShape make_box(const Vec3& he, int body, const Transform& local = Transform(),
                                   float friction = 0.5f, float restitution = 0.3f);
    static CollisionShape make_sphere(float r, int body, const Transform& local = Transform(),
                                      float friction = 0.5f, float restitution = 0.3f);
    static CollisionShape make_plane(const Vec3& normal, float offset, float friction = 0.5f,
                                     float restitution = 0.0f);
    // World box of the shape on a body at body_transform (shape.h:66-80):
    // the 8 posed corners of a box, centre +- radius of a sphere, +-1e6 for
    // a plane.
    AABB compute_aabb(const Transform& body_transform) const;
};

struct RigidBody {
    float mass = 1.0f;
    std::array<float, 9> inertia{1, 0, 0, 0, 1, 0, 0, 0, 1};  // body frame, row-major
    Vec3 com;
    float inv_mass() const { return mass > 0.0f ? 1.0f / mass : 0.0f; }
    bool is_static() const { return mass <= 0.0f; }
    std::array<float, 9> inv_inertia() const;
    static RigidBody from_box(float m, const Vec3& half_extents);
    static RigidBody from_sphere(float m, float radius);
    static RigidBody make_static();
};

struct Model {
    std::vector<RigidBody> bodies;
    std::vector<Transform> initial_transforms;
    std::vector<CollisionShape> shapes;
    int num_bodies() const { return (int)bodies.size(); }
    int num_shapes() const { return (int)shapes.size(); }
};

class ModelBuilder {
public:
    int add_body(const RigidBody& body, const Transform& transform = Transform());
    int add_shape(const CollisionShape& shape);
    int add_ground_plane(float y = 0.0f, float friction = 0.5f, float restitution = 0.0f);
    Model build() const { return model_; }
    int num_bodies() const { return model_.num_bodies(); }
    int num_shapes() const { return model_.num_shapes(); }

private:
    Model model_;
};

struct BoundaryParticle {
    Vec3 local_position;
    int body_index = -1;
    float volume = 0.0f;
};

std::vector<BoundaryParticle> sample_box_boundary(const CollisionShape& s, float spacing);
std::vector<BoundaryParticle> sample_sphere_boundary(const CollisionShape& s, float spacing);
std::vector<BoundaryParticle> sample_plane_boundary(const CollisionShape& s, float spacing,
                                                    float extent);
std::vector<BoundaryParticle> sample_model_boundaries(const Model& model, float spacing,
                                                      float plane_extent = 1.0f);

// Contact solver and sleep settings (include/novaphy/dynamics/free_body_solver.h:19-31).
struct SolverSettings {
    int velocity_iterations = 30;
    float baumgarte = 0.3f;
    float slop = 0.005f;
    bool warm_starting = true;
    bool sleep_enabled = false;
    float sleep_energy_threshold = 0.01f;
    float sleep_time_required = 0.5f;
    float sleep_ema_alpha = 0.8f;
};

// ---- rigid contacts (host; the reference's World pipeline around the fluid) ----

// One contact (include/novaphy/core/contact.h:14-35): normal from body_a
// toward body_b, penetration > 0 when overlapping; body -1 is the world.
struct ContactPoint {
    Vec3 position, normal;
    float penetration = 0.0f;
    int body_a = -1, body_b = -1, shape_a = -1, shape_b = -1;
    float friction = 0.5f, restitution = 0.0f;
    float accumulated_normal_impulse = 0.0f;
    float accumulated_tangent_impulse_1 = 0.0f, accumulated_tangent_impulse_2 = 0.0f;
};
inline float combine_friction(float a, float b) { return std::sqrt(a * b); }
inline float combine_restitution(float a, float b) { return std::max(a, b); }

// Contacts between two posed shapes, appended to `contacts`
// (src/collision/narrowphase.cpp:390-437 and the pairs before it): sphere-
// sphere, sphere-plane, box-sphere, box-plane (corners below the plane),
// box-box (15-axis SAT, up to 4 incident corners, else the midpoint).
// Returns whether the pair touches; plane-plane never does.
bool collide_shapes(const CollisionShape& a, const Transform& ta, const CollisionShape& b,
                    const Transform& tb, std::vector<ContactPoint>& contacts);

struct BroadPhasePair {
    int body_a = -1, body_b = -1;  // shape indices, body_a < body_b
    bool operator==(const BroadPhasePair& o) const { return body_a == o.body_a && body_b == o.body_b; }
};

// Broad phase (include/novaphy/collision/broadphase.h): every pair of boxes
// that overlap on all three axes (closed intervals), except pairs of two
// static shapes, as (lower, higher) index sorted lexicographically.
class SweepAndPrune {
public:
    void update(const std::vector<AABB>& aabbs, const std::vector<bool>& static_mask);
    const std::vector<BroadPhasePair>& get_pairs() const { return pairs_; }

private:
    std::vector<int> order_;
    std::vector<BroadPhasePair> pairs_;
};

struct SimState {
    std::vector<Transform> transforms;
    std::vector<Vec3> linear_velocities, angular_velocities, forces, torques;
    // Sleep bookkeeping (include/novaphy/sim/state.h): a body sleeps with its
    // whole contact island once every member's smoothed energy stayed below
    // the threshold for the required time.
    std::vector<int> sleeping;
    std::vector<float> sleep_timer, smoothed_energy;
    std::vector<int> island_id;
    void init(const std::vector<Transform>& t);
    void clear_forces();
    void set_linear_velocity(int i, const Vec3& v);
    void set_angular_velocity(int i, const Vec3& w);
    void apply_force(int i, const Vec3& f);
    void apply_torque(int i, const Vec3& t);
    void wake_body(int i);
    bool is_sleeping(int i) const;
    void update_energy(int i, float energy, float alpha);
    float get_smoothed_energy(int i) const;
    void build_islands(const std::vector<ContactPoint>& contacts);
    void evaluate_sleep(float dt, float energy_threshold, float time_threshold);
    void propagate_wake_through_island(int i);
};

// Sequential-impulse contact solver (src/dynamics/free_body_solver.cpp):
// per contact a normal row (accumulated impulse clamped at 0, Baumgarte and
// restitution bias) and two friction rows (clamped to the friction cone of
// the normal impulse), warm started from the contacts' accumulated impulses,
// velocity_iterations sweeps in contact order.
class PerformanceMonitor;
class ContactSolver {
public:
    explicit ContactSolver(SolverSettings s = {}) : settings_(s) {}
    // With a monitor, its phases world.solver.{pre_step,warm_start,
    // iteration.solve_velocity} are recorded.
    void solve(std::vector<ContactPoint>& contacts, const std::vector<RigidBody>& bodies,
               const std::vector<Transform>& transforms, std::vector<Vec3>& lin,
               std::vector<Vec3>& ang, const std::vector<int>& sleeping, float dt,
               PerformanceMonitor* monitor = nullptr);
    SolverSettings& settings() { return settings_; }
    const SolverSettings& settings() const { return settings_; }

private:
    struct Row {
        Vec3 r_a, r_b, t1, t2;
        float k_n = 0.0f, k_t1 = 0.0f, k_t2 = 0.0f;  // effective masses (inverted)
        float bias = 0.0f;
        Mat3 inv_i_a{}, inv_i_b{};  // world-frame inverse inertia
    };
    void prepare(std::vector<ContactPoint>& contacts, const std::vector<RigidBody>& bodies,
                 const std::vector<Transform>& transforms, const std::vector<Vec3>& lin,
                 const std::vector<Vec3>& ang, const std::vector<int>& sleeping, float dt);
    void sweep(std::vector<ContactPoint>& contacts, const std::vector<RigidBody>& bodies,
               std::vector<Vec3>& lin, std::vector<Vec3>& ang);
    SolverSettings settings_;
    std::vector<Row> rows_;
};

// Phase timers and per-frame metrics (include/novaphy/sim/performance_monitor.h).
struct PhaseStat {
    std::string name;
    double last_ms = 0.0, avg_ms = 0.0, max_ms = 0.0;
    int samples = 0;
};
struct MetricValue {
    std::string name;
    double value = 0.0;
};

// With trace_enabled, the phases of the last trace_frame_capacity frames are
// kept as Chrome trace events (complete events "X" for phases, counter events
// "C" for metrics) and written by write_trace_json.  Host-timed phases sit on
// thread 0 at their host time; device-timed phases (the PBF step and coupling
// phases, measured with CUDA events) on thread 1, laid end to end from the
// start of the host phase that ran them.
class PerformanceMonitor {
public:
    using Clock = std::chrono::steady_clock;
    bool enabled = false;
    bool trace_enabled = false;
    int trace_frame_capacity = 120;
    void begin_frame();
    void end_frame();
    void record_phase(const std::string& name, double ms);
    void record_phase(const std::string& name, double ms, Clock::time_point start);
    void record_device_phase(const std::string& name, double ms, double start_us);
    void record_metric(const std::string& name, double value);
    std::vector<PhaseStat> phase_stats() const;
    std::vector<MetricValue> last_frame_metrics() const { return metrics_; }
    int frame_count() const { return frames_; }
    double last_frame_total_ms() const { return last_total_ms_; }
    // Microseconds since the monitor was created (trace time stamps).
    double now_us(Clock::time_point t = Clock::now()) const;
    void write_trace_json(const std::string& path) const;
    void reset();

private:
    struct TraceEvent {
        std::string name;
        char ph = 'X';
        double ts_us = 0.0, dur_us = 0.0, value = 0.0;
        int tid = 0;
    };
    bool tracing() const { return enabled && trace_enabled; }
    void stat(const std::string& name, double ms);
    std::map<std::string, PhaseStat> phases_;
    std::vector<MetricValue> metrics_, pending_;
    int frames_ = 0;
    double last_total_ms_ = 0.0;
    Clock::time_point frame_start_{};
    Clock::time_point epoch_ = Clock::now();
    std::vector<TraceEvent> trace_cur_;
    std::vector<std::vector<TraceEvent>> trace_frames_;  // oldest first
};

// Rigid world (src/sim/world.cpp:30-182): symplectic Euler velocity update
// (src/dynamics/integrator.cpp:20-60), shape boxes, broad phase, narrow
// phase, contact islands and sleep (when enabled), the contact solver,
// position update, forces cleared.
class World {
public:
    explicit World(const Model& model, SolverSettings settings = {});
    virtual ~World() = default;
    void step(float dt);
    void set_gravity(const Vec3& g) { gravity_ = g; }
    const Vec3& gravity() const { return gravity_; }
    SimState& state() { return state_; }
    const Model& model() const { return model_; }
    const std::vector<ContactPoint>& contacts() const { return contacts_; }
    SolverSettings& solver_settings() { return solver_.settings(); }
    PerformanceMonitor& performance_monitor() { return monitor_; }
    // Forces and torques last one step; with sleep on they wake the body.
    void apply_force(int body, const Vec3& f);
    void apply_torque(int body, const Vec3& t);

protected:
    void step_rigid_pipeline(float dt);
    // m |v|^2 + w . (I w): twice the kinetic energy, the sleep test's measure.
    float kinetic_energy(int body) const;
    Model model_;
    ContactSolver solver_;
    SimState state_;
    SweepAndPrune broadphase_;
    std::vector<ContactPoint> contacts_;
    Vec3 gravity_{0.0f, -9.81f, 0.0f};  // include/novaphy/sim/world.h:157
    PerformanceMonitor monitor_;
};

// PBFSolver (include/novaphy/fluid/pbf_solver.h:52-116): the step runs on the
// device; the ParticleState stays on the host and is copied each call.
class PBFSolver {
public:
    explicit PBFSolver(const PBFSettings& settings = {}) : settings_(settings) {}
    ~PBFSolver();
    PBFSolver(const PBFSolver&) = delete;
    PBFSolver& operator=(const PBFSolver&) = delete;
    void step(ParticleState& state, float dt, const Vec3& gravity, float particle_mass);
    PBFSettings& settings() { return settings_; }

private:
    PBFSettings settings_;
    pbf_scene* scene_ = nullptr;
};

// FluidWorld (include/novaphy/fluid/fluid_world.h): device-resident fluid and
// Akinci boundary, host rigid bodies.
class FluidWorld : public World {
public:
    FluidWorld(const Model& model, const std::vector<FluidBlockDef>& blocks = {},
               SolverSettings solver_settings = {}, PBFSettings pbf_settings = {},
               float boundary_extent = 1.0f);
    ~FluidWorld() override;
    void step(float dt);
    ParticleState& fluid_state();
    PBFSettings& pbf_settings() { return pbf_; }
    int num_particles() const { return n_; }
    int num_boundary_particles() const { return (int)boundary_.size(); }
    const std::vector<BoundaryParticle>& boundary_particles() const { return boundary_; }
    // Zero-copy state access (no counterpart in the reference, whose
    // accessors copy).  fluid_pinned(field): the field (PBF_FIELD_*) read by
    // one DMA into page-locked host memory that the world owns, 3n floats for
    // positions and velocities, n for densities and lambdas; it is re-read
    // only when a step ran since the last read of that field, and stays valid
    // until the world is destroyed (later reads overwrite it).
    // fluid_device_field(field): the device pointer of the field (float4 rows
    // for positions and velocities, floats otherwise) once the scene's stream
    // is idle; valid until the world is destroyed.
    const float* fluid_pinned(int field);
    void* fluid_device_field(int field);

private:
    struct PinnedField {
        float* p = nullptr;
        size_t floats = 0;
        bool stale = true;
    };
    PinnedField pinned_[4];
    PBFSettings pbf_;
    std::vector<BoundaryParticle> boundary_;
    ParticleState host_;
    bool host_dirty_ = false;
    int n_ = 0;
    float particle_mass_ = 0.0f;
    float spacing_ = 0.02f;
    pbf_scene* scene_ = nullptr;
};

// Throws std::invalid_argument for PBF_ERR_INVALID_ARG, std::runtime_error otherwise.
void check_pbf(int rc);

}  // namespace novaphy_gb300
