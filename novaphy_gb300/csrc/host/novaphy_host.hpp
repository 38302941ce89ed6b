// Host layer of the GB300 PBF path: NovaPhy's fluid API (the types of
// include/novaphy/fluid/*.h and the parts of sim/core/math they use) on top
// of the C ABI in include/novaphy_pbf.h.  The PBF step, the neighbour search
// and the Akinci coupling run on the device; setup (fluid blocks, boundary
// sampling) and the small rigid-body state stay on the host.
#pragma once

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
    Vec3& operator+=(const Vec3& o) {
        x = x + o.x;
        y = y + o.y;
        z = z + o.z;
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

// Unit quaternion (w, x, y, z).
struct Quat {
    float w = 1.0f, x = 0.0f, y = 0.0f, z = 0.0f;
    Vec3 vec() const { return {x, y, z}; }
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
    Vec3 transform_point(const Vec3& p) const { return position + rotation.rotate(p); }
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

struct SolverSettings {
    int velocity_iterations = 20;
    float baumgarte = 0.2f;
    float slop = 0.005f;
    bool warm_starting = true;
    bool sleep_enabled = false;
};

struct SimState {
    std::vector<Transform> transforms;
    std::vector<Vec3> linear_velocities, angular_velocities, forces, torques;
    void init(const std::vector<Transform>& t);
    void set_linear_velocity(int i, const Vec3& v);
    void set_angular_velocity(int i, const Vec3& w);
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

// Rigid world: gravity, accumulated forces, symplectic Euler integration
// (src/dynamics/integrator.cpp:20-60).  Contacts are not modelled here.
class World {
public:
    explicit World(const Model& model, SolverSettings settings = {});
    virtual ~World() = default;
    void step(float dt);
    void set_gravity(const Vec3& g) { gravity_ = g; }
    const Vec3& gravity() const { return gravity_; }
    SimState& state() { return state_; }
    const Model& model() const { return model_; }
    PerformanceMonitor& performance_monitor() { return monitor_; }
    void apply_force(int body, const Vec3& f);
    void apply_torque(int body, const Vec3& t);

protected:
    void step_rigid_pipeline(float dt);
    Model model_;
    SolverSettings settings_;
    SimState state_;
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

private:
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
