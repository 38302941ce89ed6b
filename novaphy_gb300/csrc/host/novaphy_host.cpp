// Host layer implementation (see novaphy_host.hpp).  Compiled with
// -ffp-contract=off so that host float arithmetic rounds like the reference.
#include "novaphy_host.hpp"
#include "rigid_step.hpp"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <fstream>

namespace novaphy_gb300 {

void check_pbf(int rc) {
    if (rc == PBF_OK) return;
    const char* m = pbf_last_error();
    const std::string msg = m ? m : "unknown error";
    if (rc == PBF_ERR_INVALID_ARG) throw std::invalid_argument(msg);
    throw std::runtime_error("novaphy_gb300: " + msg);
}

static int device_index() {
    const char* e = std::getenv("NOVAPHY_GB300_DEVICE");
    return e ? std::atoi(e) : 0;
}

::pbf_settings PBFSettings::to_c() const {
    ::pbf_settings s;
    pbf_default_settings(&s);
    s.rest_density = rest_density;
    s.kernel_radius = kernel_radius;
    s.particle_radius = particle_radius;
    s.solver_iterations = solver_iterations;
    s.epsilon = epsilon;
    s.xsph_viscosity = xsph_viscosity;
    s.vorticity_epsilon = vorticity_epsilon;
    s.corr_delta_q = corr_delta_q;
    s.corr_k = corr_k;
    s.corr_n = corr_n;
    s.use_domain_bounds = use_domain_bounds ? 1 : 0;
    for (int d = 0; d < 3; ++d) {
        s.domain_lower[d] = domain_lower[d];
        s.domain_upper[d] = domain_upper[d];
    }
    s.exact_arithmetic = exact_arithmetic ? 1 : 0;
    s.hash_compat = hash_compat ? 1 : 0;
    s.boundary_two_way = boundary_two_way ? 1 : 0;
    s.boundary_friction = boundary_friction;
    return s;
}

// ---- SPH kernels (sph_kernel.h:24-80) ----

float SPHKernels::poly6(float r_sq, float h) {
    if (r_sq >= h * h) return 0.0f;
    const float h2 = h * h;
    const float diff = h2 - r_sq;
    const float h9 = h2 * h2 * h2 * h2 * h;
    return (315.0f / (64.0f * kPi * h9)) * diff * diff * diff;
}

Vec3 SPHKernels::spiky_grad(const Vec3& r, float h) {
    const float r_len = r.norm();
    if (r_len <= 1e-7f || r_len >= h) return Vec3{};
    const float diff = h - r_len;
    const float h6 = h * h * h * h * h * h;
    const float coeff = -(45.0f / (kPi * h6)) * diff * diff / r_len;
    return coeff * r;
}

float SPHKernels::spiky(float r_len, float h) {
    if (r_len >= h || r_len < 0.0f) return 0.0f;
    const float diff = h - r_len;
    const float h6 = h * h * h * h * h * h;
    return (15.0f / (kPi * h6)) * diff * diff * diff;
}

float SPHKernels::cubic_spline(float r_len, float h) {
    const float q = r_len / h;
    if (q >= 1.0f) return 0.0f;
    const float h3 = h * h * h;
    const float sigma = 8.0f / (kPi * h3);
    if (q <= 0.5f) return sigma * (6.0f * (q * q * q - q * q) + 1.0f);
    const float t = 1.0f - q;
    return sigma * 2.0f * t * t * t;
}

// ---- particles ----

std::vector<Vec3> generate_fluid_block(const FluidBlockDef& def) {
    std::vector<Vec3> out;
    const float s = def.particle_spacing;
    if (s <= 0.0f) return out;
    int n[3];
    for (int d = 0; d < 3; ++d)
        n[d] = std::max(1, (int)std::floor((def.upper[d] - def.lower[d]) / s) + 1);
    out.reserve((size_t)n[0] * n[1] * n[2]);
    for (int iz = 0; iz < n[2]; ++iz)
        for (int iy = 0; iy < n[1]; ++iy)
            for (int ix = 0; ix < n[0]; ++ix)
                out.emplace_back(def.lower.x + (float)ix * s, def.lower.y + (float)iy * s,
                                 def.lower.z + (float)iz * s);
    return out;
}

void ParticleState::init(const std::vector<Vec3>& p, const Vec3& v0) {
    positions = p;
    velocities.assign(p.size(), v0);
    densities.assign(p.size(), 0.0f);
    lambdas.assign(p.size(), 0.0f);
}

void ParticleState::clear() {
    positions.clear();
    velocities.clear();
    densities.clear();
    lambdas.clear();
}

// ---- host hash grid (neighbor_search.cpp) ----

uint64_t SpatialHashGrid::hash_cell(int cx, int cy, int cz) {
    return ((uint64_t)(int64_t)cx * 73856093ULL) ^ ((uint64_t)(int64_t)cy * 19349663ULL) ^
           ((uint64_t)(int64_t)cz * 83492791ULL);
}

void SpatialHashGrid::world_to_cell(const Vec3& p, int& cx, int& cy, int& cz) const {
    const float inv = 1.0f / cell_size_;
    cx = (int)std::floor(p.x * inv);
    cy = (int)std::floor(p.y * inv);
    cz = (int)std::floor(p.z * inv);
}

void SpatialHashGrid::build(const std::vector<Vec3>& positions) {
    cells_.clear();
    for (size_t i = 0; i < positions.size(); ++i) {
        int cx, cy, cz;
        world_to_cell(positions[i], cx, cy, cz);
        cells_[hash_cell(cx, cy, cz)].push_back((int)i);
    }
}

std::vector<int> SpatialHashGrid::query_neighbors(const Vec3& point, float) const {
    std::vector<int> out;
    int cx, cy, cz;
    world_to_cell(point, cx, cy, cz);
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                auto it = cells_.find(hash_cell(cx + dx, cy + dy, cz + dz));
                if (it != cells_.end()) out.insert(out.end(), it->second.begin(), it->second.end());
            }
    return out;
}

std::vector<std::pair<int, int>> SpatialHashGrid::query_all_pairs(const std::vector<Vec3>& pos,
                                                                  float radius) const {
    std::vector<std::pair<int, int>> pairs;
    const float r2 = radius * radius;
    for (size_t i = 0; i < pos.size(); ++i)
        for (int j : query_neighbors(pos[i], radius))
            if (j > (int)i && (pos[i] - pos[(size_t)j]).squaredNorm() < r2)
                pairs.emplace_back((int)i, j);
    return pairs;
}

// ---- rigid model ----

CollisionShape CollisionShape::make_box(const Vec3& he, int body, const Transform& local,
                                        float friction, float restitution) {
    CollisionShape s;
    s.type = ShapeType::Box;
    s.half_extents = he;
    s.body_index = body;
    s.local_transform = local;
    s.friction = friction;
    s.restitution = restitution;
    return s;
}

CollisionShape CollisionShape::make_sphere(float r, int body, const Transform& local,
                                           float friction, float restitution) {
    CollisionShape s;
    s.type = ShapeType::Sphere;
    s.radius = r;
    s.body_index = body;
    s.local_transform = local;
    s.friction = friction;
    s.restitution = restitution;
    return s;
}

CollisionShape CollisionShape::make_plane(const Vec3& normal, float offset, float friction,
                                          float restitution) {
    CollisionShape s;
    s.type = ShapeType::Plane;
    s.normal = normal.normalized();
    s.offset = offset;
    s.body_index = -1;
    s.friction = friction;
    s.restitution = restitution;
    return s;
}

std::array<float, 9> RigidBody::inv_inertia() const {
    std::array<float, 9> r{};
    if (mass <= 0.0f) return r;
    const auto& a = inertia;
    const float det = a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
                      a[2] * (a[3] * a[7] - a[4] * a[6]);
    if (det == 0.0f) return r;
    const float id = 1.0f / det;
    r[0] = (a[4] * a[8] - a[5] * a[7]) * id;
    r[1] = (a[2] * a[7] - a[1] * a[8]) * id;
    r[2] = (a[1] * a[5] - a[2] * a[4]) * id;
    r[3] = (a[5] * a[6] - a[3] * a[8]) * id;
    r[4] = (a[0] * a[8] - a[2] * a[6]) * id;
    r[5] = (a[2] * a[3] - a[0] * a[5]) * id;
    r[6] = (a[3] * a[7] - a[4] * a[6]) * id;
    r[7] = (a[1] * a[6] - a[0] * a[7]) * id;
    r[8] = (a[0] * a[4] - a[1] * a[3]) * id;
    return r;
}

RigidBody RigidBody::from_box(float m, const Vec3& he) {
    RigidBody b;
    b.mass = m;
    const float w = 2.0f * he.x, h = 2.0f * he.y, d = 2.0f * he.z, c = m / 12.0f;
    b.inertia = {c * (h * h + d * d), 0, 0, 0, c * (w * w + d * d), 0, 0, 0, c * (w * w + h * h)};
    return b;
}

RigidBody RigidBody::from_sphere(float m, float r) {
    RigidBody b;
    b.mass = m;
    const float I = (2.0f / 5.0f) * m * r * r;
    b.inertia = {I, 0, 0, 0, I, 0, 0, 0, I};
    return b;
}

RigidBody RigidBody::make_static() {
    RigidBody b;
    b.mass = 0.0f;
    b.inertia = {};
    return b;
}

int ModelBuilder::add_body(const RigidBody& body, const Transform& t) {
    model_.bodies.push_back(body);
    model_.initial_transforms.push_back(t);
    return (int)model_.bodies.size() - 1;
}

int ModelBuilder::add_shape(const CollisionShape& s) {
    model_.shapes.push_back(s);
    return (int)model_.shapes.size() - 1;
}

int ModelBuilder::add_ground_plane(float y, float friction, float restitution) {
    return add_shape(CollisionShape::make_plane(Vec3{0.0f, 1.0f, 0.0f}, y, friction, restitution));
}

// ---- boundary sampling (src/fluid/boundary.cpp:15-150) ----

std::vector<BoundaryParticle> sample_box_boundary(const CollisionShape& s, float spacing) {
    std::vector<BoundaryParticle> out;
    if (s.type != ShapeType::Box) return out;
    const Vec3& he = s.half_extents;
    for (int axis = 0; axis < 3; ++axis) {
        const int a1 = (axis + 1) % 3, a2 = (axis + 2) % 3;
        const int n1 = std::max(1, (int)std::floor(2.0f * he[a1] / spacing) + 1);
        const int n2 = std::max(1, (int)std::floor(2.0f * he[a2] / spacing) + 1);
        for (int sign = -1; sign <= 1; sign += 2)
            for (int i1 = 0; i1 < n1; ++i1)
                for (int i2 = 0; i2 < n2; ++i2) {
                    Vec3 lp;
                    lp[axis] = (float)sign * he[axis];
                    lp[a1] = -he[a1] + (float)i1 * spacing;
                    lp[a2] = -he[a2] + (float)i2 * spacing;
                    out.push_back({s.local_transform.transform_point(lp), s.body_index, 0.0f});
                }
    }
    return out;
}

std::vector<BoundaryParticle> sample_sphere_boundary(const CollisionShape& s, float spacing) {
    std::vector<BoundaryParticle> out;
    if (s.type != ShapeType::Sphere) return out;
    const float r = s.radius;
    const float area = 4.0f * kPi * r * r;
    const int n = std::max(12, (int)(area / (spacing * spacing)));
    const float golden_ratio = (1.0f + std::sqrt(5.0f)) / 2.0f;
    const float golden_angle = 2.0f * kPi / (golden_ratio * golden_ratio);
    for (int i = 0; i < n; ++i) {
        const float theta = std::acos(1.0f - 2.0f * ((float)i + 0.5f) / (float)n);
        const float phi = golden_angle * (float)i;
        const Vec3 lp(r * std::sin(theta) * std::cos(phi), r * std::sin(theta) * std::sin(phi),
                      r * std::cos(theta));
        out.push_back({s.local_transform.transform_point(lp), s.body_index, 0.0f});
    }
    return out;
}

std::vector<BoundaryParticle> sample_plane_boundary(const CollisionShape& s, float spacing,
                                                    float extent) {
    std::vector<BoundaryParticle> out;
    if (s.type != ShapeType::Plane) return out;
    const Vec3& nrm = s.normal;
    const Vec3 t1 = (std::fabs(nrm.y) < 0.9f ? Vec3(0, 1, 0).cross(nrm) : Vec3(1, 0, 0).cross(nrm))
                        .normalized();
    const Vec3 t2 = nrm.cross(t1).normalized();
    const int n = (int)std::floor(2.0f * extent / spacing) + 1;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            const float a = -extent + (float)i * spacing;
            const float b = -extent + (float)j * spacing;
            out.push_back({(nrm * s.offset + t1 * a) + t2 * b, s.body_index, 0.0f});
        }
    return out;
}

std::vector<BoundaryParticle> sample_model_boundaries(const Model& model, float spacing,
                                                      float plane_extent) {
    std::vector<BoundaryParticle> all;
    for (const auto& s : model.shapes) {
        std::vector<BoundaryParticle> p;
        switch (s.type) {
            case ShapeType::Box: p = sample_box_boundary(s, spacing); break;
            case ShapeType::Sphere: p = sample_sphere_boundary(s, spacing); break;
            case ShapeType::Plane: p = sample_plane_boundary(s, spacing, plane_extent); break;
        }
        all.insert(all.end(), p.begin(), p.end());
    }
    return all;
}

// ---- world ----

void PerformanceMonitor::begin_frame() {
    pending_.clear();
    trace_cur_.clear();
    frame_start_ = Clock::now();
}

void PerformanceMonitor::end_frame() {
    if (!enabled) return;
    const Clock::time_point t = Clock::now();
    last_total_ms_ = std::chrono::duration<double, std::milli>(t - frame_start_).count();
    metrics_ = pending_;
    ++frames_;
    if (tracing()) {
        const double ts = now_us(t);
        for (const MetricValue& m : metrics_) {
            TraceEvent e;
            e.name = m.name;
            e.ph = 'C';
            e.ts_us = ts;
            e.value = m.value;
            trace_cur_.push_back(e);
        }
        trace_frames_.push_back(std::move(trace_cur_));
        trace_cur_.clear();
        const size_t cap = (size_t)std::max(trace_frame_capacity, 1);
        if (trace_frames_.size() > cap)
            trace_frames_.erase(trace_frames_.begin(),
                                trace_frames_.begin() + (long)(trace_frames_.size() - cap));
    }
}

double PerformanceMonitor::now_us(Clock::time_point t) const {
    return std::chrono::duration<double, std::micro>(t - epoch_).count();
}

void PerformanceMonitor::stat(const std::string& name, double ms) {
    PhaseStat& p = phases_[name];
    p.name = name;
    p.last_ms = ms;
    p.max_ms = std::max(p.max_ms, ms);
    p.avg_ms = (p.avg_ms * p.samples + ms) / (p.samples + 1);
    ++p.samples;
}

void PerformanceMonitor::record_phase(const std::string& name, double ms) {
    record_phase(name, ms, Clock::now() - std::chrono::duration_cast<Clock::duration>(
                                              std::chrono::duration<double, std::milli>(ms)));
}

void PerformanceMonitor::record_phase(const std::string& name, double ms, Clock::time_point start) {
    if (!enabled) return;
    stat(name, ms);
    if (tracing()) {
        TraceEvent e;
        e.name = name;
        e.ts_us = now_us(start);
        e.dur_us = ms * 1e3;
        trace_cur_.push_back(e);
    }
}

void PerformanceMonitor::record_device_phase(const std::string& name, double ms, double start_us) {
    if (!enabled) return;
    stat(name, ms);
    if (tracing()) {
        TraceEvent e;
        e.name = name;
        e.ts_us = start_us;
        e.dur_us = ms * 1e3;
        e.tid = 1;
        trace_cur_.push_back(e);
    }
}

namespace {
std::string json_escape(const std::string& s) {
    std::string o;
    for (char c : s) {
        if (c == '"' || c == '\\') {
            o += '\\';
            o += c;
        } else if ((unsigned char)c < 0x20) {
            char buf[8];
            std::snprintf(buf, sizeof(buf), "\\u%04x", (unsigned)(unsigned char)c);
            o += buf;
        } else {
            o += c;
        }
    }
    return o;
}
}  // namespace

void PerformanceMonitor::write_trace_json(const std::string& path) const {
    std::ofstream out(path);
    if (!out) throw std::runtime_error("cannot write the trace file " + path);
    out.precision(17);
    out << "{\"traceEvents\": [";
    bool first = true;
    for (const auto& frame : trace_frames_)
        for (const TraceEvent& e : frame) {
            out << (first ? "\n" : ",\n");
            first = false;
            out << "{\"name\": \"" << json_escape(e.name) << "\", \"ph\": \"" << e.ph
                << "\", \"ts\": " << e.ts_us << ", \"pid\": 0, \"tid\": " << e.tid;
            if (e.ph == 'X') out << ", \"dur\": " << e.dur_us << ", \"cat\": \"novaphy\"";
            else out << ", \"args\": {\"value\": " << e.value << "}";
            out << "}";
        }
    out << (first ? "" : "\n") << "], \"displayTimeUnit\": \"ms\"}\n";
    if (!out) throw std::runtime_error("writing the trace file " + path + " failed");
}

void PerformanceMonitor::record_metric(const std::string& name, double value) {
    if (!enabled) return;
    pending_.push_back({name, value});
}

std::vector<PhaseStat> PerformanceMonitor::phase_stats() const {
    std::vector<PhaseStat> out;
    for (const auto& kv : phases_) out.push_back(kv.second);
    return out;
}

void PerformanceMonitor::reset() {
    phases_.clear();
    metrics_.clear();
    pending_.clear();
    frames_ = 0;
    last_total_ms_ = 0.0;
    trace_cur_.clear();
    trace_frames_.clear();
}

namespace {
struct Scope {
    PerformanceMonitor& m;
    std::string name;
    PerformanceMonitor::Clock::time_point t0 = PerformanceMonitor::Clock::now();
    Scope(PerformanceMonitor& mon, const char* n) : m(mon), name(n) {}
    ~Scope() {
        m.record_phase(name,
                       std::chrono::duration<double, std::milli>(
                           PerformanceMonitor::Clock::now() - t0)
                           .count(),
                       t0);
    }
};
}  // namespace

World::World(const Model& model, SolverSettings settings) : model_(model), solver_(settings) {
    for (const CollisionShape& sh : model_.shapes)
        if (sh.body_index >= model_.num_bodies())
            throw std::invalid_argument("shape refers to a body the model does not have");
    state_.init(model_.initial_transforms);
}

// With sleep on, a force or torque first wakes a sleeping body (at rest, its
// island with it), world.cpp:184-218.
void World::apply_force(int i, const Vec3& f) {
    if (solver_.settings().sleep_enabled && state_.is_sleeping(i)) state_.wake_body(i);
    state_.apply_force(i, f);
}

void World::apply_torque(int i, const Vec3& t) {
    if (solver_.settings().sleep_enabled && state_.is_sleeping(i)) state_.wake_body(i);
    state_.apply_torque(i, t);
}

void World::step(float dt) {
    monitor_.begin_frame();
    step_rigid_pipeline(dt);
    monitor_.end_frame();
}

float World::kinetic_energy(int i) const {
    const RigidBody& b = model_.bodies[(size_t)i];
    const Vec3& v = state_.linear_velocities[(size_t)i];
    const Vec3& w = state_.angular_velocities[(size_t)i];
    const auto& I = b.inertia;
    const Vec3 iw(I[0] * w.x + (I[1] * w.y + I[2] * w.z), I[3] * w.x + (I[4] * w.y + I[5] * w.z),
                  I[6] * w.x + (I[7] * w.y + I[8] * w.z));
    return b.mass * v.squaredNorm() + w.dot(iw);
}

// The reference's step order (world.cpp:30-182); sleeping bodies neither
// integrate nor move, and count as static in the broad phase.
void World::step_rigid_pipeline(float dt) {
    Scope total(monitor_, "world.total");
    const int n = model_.num_bodies();
    const SolverSettings& set = solver_.settings();
    const bool sleep = set.sleep_enabled;
    int dynamic = 0;
    {
        Scope s(monitor_, "world.integrate_velocity");
        for (int i = 0; i < n; ++i) {
            const RigidBody& b = model_.bodies[(size_t)i];
            if (b.is_static() || (sleep && state_.is_sleeping(i))) continue;
            ++dynamic;
            Vec3& v = state_.linear_velocities[(size_t)i];
            Vec3& w = state_.angular_velocities[(size_t)i];
            const float g[3] = {gravity_.x, gravity_.y, gravity_.z};
            const Vec3& f = state_.forces[(size_t)i];
            const Vec3& t = state_.torques[(size_t)i];
            const float fa[3] = {f.x, f.y, f.z}, ta[3] = {t.x, t.y, t.z};
            float va[3] = {v.x, v.y, v.z}, wa[3] = {w.x, w.y, w.z};
            const auto ii = b.inv_inertia();
            pbf_rigid::integrate_velocity(va, wa, g, fa, b.inv_mass(), ii.data(), ta, dt);
            v = Vec3(va[0], va[1], va[2]);
            w = Vec3(wa[0], wa[1], wa[2]);
            if (sleep) state_.update_energy(i, kinetic_energy(i), set.sleep_ema_alpha);
        }
    }
    const int ns = model_.num_shapes();
    std::vector<AABB> boxes((size_t)ns);
    std::vector<bool> fixed((size_t)ns);
    {
        Scope s(monitor_, "world.broadphase.build_aabbs");
        for (int k = 0; k < ns; ++k) {
            const CollisionShape& sh = model_.shapes[(size_t)k];
            if (sh.body_index >= 0) {
                boxes[(size_t)k] = sh.compute_aabb(state_.transforms[(size_t)sh.body_index]);
                fixed[(size_t)k] = model_.bodies[(size_t)sh.body_index].is_static() ||
                                   (sleep && state_.is_sleeping(sh.body_index));
            } else {
                boxes[(size_t)k] = sh.compute_aabb(Transform::identity());
                fixed[(size_t)k] = true;
            }
        }
    }
    {
        Scope s(monitor_, "world.broadphase.sap");
        broadphase_.update(boxes, fixed);
    }
    contacts_.clear();
    {
        Scope s(monitor_, "world.narrowphase.total");
        std::vector<ContactPoint> found;
        for (const BroadPhasePair& p : broadphase_.get_pairs()) {
            const CollisionShape& sa = model_.shapes[(size_t)p.body_a];
            const CollisionShape& sb = model_.shapes[(size_t)p.body_b];
            const Transform ta =
                sa.body_index >= 0 ? state_.transforms[(size_t)sa.body_index] : Transform::identity();
            const Transform tb =
                sb.body_index >= 0 ? state_.transforms[(size_t)sb.body_index] : Transform::identity();
            found.clear();
            if (!collide_shapes(sa, ta, sb, tb, found)) continue;
            for (ContactPoint& c : found) {
                c.friction = combine_friction(sa.friction, sb.friction);
                c.restitution = combine_restitution(sa.restitution, sb.restitution);
                contacts_.push_back(c);
            }
        }
    }
    if (sleep) {
        Scope s(monitor_, "world.build_islands");
        state_.build_islands(contacts_);
    }
    {
        Scope s(monitor_, "world.solver.total");
        solver_.solve(contacts_, model_.bodies, state_.transforms, state_.linear_velocities,
                      state_.angular_velocities, state_.sleeping, dt, &monitor_);
    }
    if (sleep) {
        {
            // an awake body touching a sleeping one wakes the sleeper's island
            Scope s(monitor_, "world.propagate_wakes");
            for (const ContactPoint& c : contacts_) {
                const bool a = c.body_a >= 0 && state_.is_sleeping(c.body_a);
                const bool b = c.body_b >= 0 && state_.is_sleeping(c.body_b);
                if (a && !b) state_.propagate_wake_through_island(c.body_a);
                else if (!a && b) state_.propagate_wake_through_island(c.body_b);
            }
        }
        Scope s(monitor_, "world.evaluate_sleep");
        state_.evaluate_sleep(dt, set.sleep_energy_threshold, set.sleep_time_required);
    }
    {
        Scope s(monitor_, "world.integrate_position");
        for (int i = 0; i < n; ++i) {
            if (model_.bodies[(size_t)i].is_static() || (sleep && state_.is_sleeping(i))) continue;
            Transform& tr = state_.transforms[(size_t)i];
            const Vec3& v = state_.linear_velocities[(size_t)i];
            const Vec3& w = state_.angular_velocities[(size_t)i];
            float p[3] = {tr.position.x, tr.position.y, tr.position.z};
            float q[4] = {tr.rotation.w, tr.rotation.x, tr.rotation.y, tr.rotation.z};
            const float va[3] = {v.x, v.y, v.z}, wa[3] = {w.x, w.y, w.z};
            pbf_rigid::integrate_position(p, q, va, wa, dt);
            tr.position = Vec3(p[0], p[1], p[2]);
            tr.rotation = Quat{q[0], q[1], q[2], q[3]};
        }
    }
    {
        Scope s(monitor_, "world.clear_forces");
        state_.clear_forces();
    }
    monitor_.record_metric("bodies", (double)n);
    monitor_.record_metric("dynamic_bodies", (double)dynamic);
    monitor_.record_metric("shapes", (double)ns);
    monitor_.record_metric("candidate_pairs", (double)broadphase_.get_pairs().size());
    monitor_.record_metric("contacts", (double)contacts_.size());
    monitor_.record_metric("solver_iterations", (double)set.velocity_iterations);
}

// ---- PBFSolver ----

PBFSolver::~PBFSolver() {
    if (scene_) pbf_scene_destroy(scene_);
}

void PBFSolver::step(ParticleState& st, float dt, const Vec3& g, float mass) {
    const int n = st.num_particles();
    if (n == 0) return;  // pbf_solver.cpp:21
    const ::pbf_settings s = settings_.to_c();
    if (!scene_) check_pbf(pbf_scene_create(device_index(), &s, 0, nullptr, nullptr, mass, &scene_));
    else check_pbf(pbf_scene_set_settings(scene_, &s));
    st.velocities.resize((size_t)n);
    st.densities.resize((size_t)n, 0.0f);
    st.lambdas.resize((size_t)n, 0.0f);
    const float g3[3] = {g.x, g.y, g.z};
    check_pbf(pbf_solver_step_host(scene_, n, &st.positions[0].x, &st.velocities[0].x,
                                   st.densities.data(), st.lambdas.data(), dt, g3, mass));
}

// ---- FluidWorld ----

FluidWorld::FluidWorld(const Model& model, const std::vector<FluidBlockDef>& blocks,
                       SolverSettings solver_settings, PBFSettings pbf_settings,
                       float boundary_extent)
    : World(model, solver_settings), pbf_(pbf_settings) {
    std::vector<Vec3> pos;
    Vec3 v0;
    for (const auto& b : blocks) {  // fluid_world.cpp:23-29: the last block's v0 and spacing
        auto p = generate_fluid_block(b);
        pos.insert(pos.end(), p.begin(), p.end());
        v0 = b.initial_velocity;
        spacing_ = b.particle_spacing;
    }
    n_ = (int)pos.size();
    if (n_ > 0) {
        host_.init(pos, v0);
        particle_mass_ = pbf_.particle_mass(spacing_);
    }
    boundary_ = sample_model_boundaries(model_, spacing_, boundary_extent);
    if (n_ == 0 && boundary_.empty()) return;
    const ::pbf_settings s = pbf_.to_c();
    std::vector<Vec3> vel(pos.size(), v0);
    check_pbf(pbf_scene_create(device_index(), &s, n_, n_ ? &pos[0].x : nullptr,
                               n_ ? &vel[0].x : nullptr, particle_mass_, &scene_));
    if (!boundary_.empty()) {
        // Akinci volumes at the initial poses, over all boundary particles together.
        std::vector<Vec3> world(boundary_.size());
        for (size_t i = 0; i < boundary_.size(); ++i) {
            const int bi = boundary_[i].body_index;
            world[i] = (bi >= 0 && bi < (int)state_.transforms.size())
                           ? state_.transforms[(size_t)bi].transform_point(boundary_[i].local_position)
                           : boundary_[i].local_position;
        }
        std::vector<float> psi(boundary_.size());
        check_pbf(pbf_boundary_volumes(device_index(), (int)world.size(), &world[0].x,
                                       pbf_.kernel_radius, psi.data()));
        std::vector<Vec3> local(boundary_.size());
        std::vector<int> body(boundary_.size());
        for (size_t i = 0; i < boundary_.size(); ++i) {
            boundary_[i].volume = psi[i];
            local[i] = boundary_[i].local_position;
            body[i] = boundary_[i].body_index;
        }
        check_pbf(pbf_scene_set_boundary(scene_, (int)boundary_.size(), &local[0].x, body.data(),
                                         psi.data()));
    }
}

FluidWorld::~FluidWorld() {
    for (auto& f : pinned_) pbf_host_free(f.p);
    if (scene_) pbf_scene_destroy(scene_);
}

const float* FluidWorld::fluid_pinned(int field) {
    if (field < PBF_FIELD_POSITIONS || field > PBF_FIELD_LAMBDAS)
        throw std::invalid_argument("unknown fluid field");
    PinnedField& f = pinned_[field];
    const bool vec = field == PBF_FIELD_POSITIONS || field == PBF_FIELD_VELOCITIES;
    const size_t floats = (size_t)n_ * (vec ? 3 : 1);
    if (floats == 0) return nullptr;
    if (!f.p || f.floats != floats) {
        pbf_host_free(f.p);
        f.p = nullptr;
        void* p = nullptr;
        check_pbf(pbf_host_alloc(floats * sizeof(float), &p));
        f.p = static_cast<float*>(p);
        f.floats = floats;
        f.stale = true;
    }
    if (f.stale && scene_) {
        check_pbf(pbf_scene_read(scene_, field, f.p));
    } else if (f.stale) {
        // No device scene (no particles): nothing to read.
        std::fill(f.p, f.p + floats, 0.0f);
    }
    f.stale = false;
    return f.p;
}

void* FluidWorld::fluid_device_field(int field) {
    if (field < PBF_FIELD_POSITIONS || field > PBF_FIELD_LAMBDAS)
        throw std::invalid_argument("unknown fluid field");
    if (!scene_ || n_ == 0) return nullptr;
    void* p = nullptr;
    check_pbf(pbf_scene_device_field(scene_, field, &p));
    check_pbf(pbf_scene_sync(scene_));
    return p;
}

ParticleState& FluidWorld::fluid_state() {
    if (host_dirty_ && scene_ && n_ > 0) {
        host_.positions.resize((size_t)n_);
        host_.velocities.resize((size_t)n_);
        host_.densities.resize((size_t)n_);
        host_.lambdas.resize((size_t)n_);
        check_pbf(pbf_scene_read(scene_, PBF_FIELD_POSITIONS, &host_.positions[0].x));
        check_pbf(pbf_scene_read(scene_, PBF_FIELD_VELOCITIES, &host_.velocities[0].x));
        check_pbf(pbf_scene_read(scene_, PBF_FIELD_DENSITIES, host_.densities.data()));
        check_pbf(pbf_scene_read(scene_, PBF_FIELD_LAMBDAS, host_.lambdas.data()));
        host_dirty_ = false;
    }
    return host_;
}

void FluidWorld::step(float dt) {
    monitor_.begin_frame();
    {
        Scope total(monitor_, "fluid.total");
        if (n_ > 0 && scene_) {
            const ::pbf_settings s = pbf_.to_c();
            check_pbf(pbf_scene_set_settings(scene_, &s));
            const float g3[3] = {gravity_.x, gravity_.y, gravity_.z};
            check_pbf(pbf_scene_set_gravity(scene_, g3));
            check_pbf(pbf_scene_set_mass(scene_, particle_mass_));
            int needed = 0;
            for (const auto& b : boundary_) needed = std::max(needed, b.body_index + 1);
            std::vector<float> pos(3 * (size_t)needed), quat(4 * (size_t)needed);
            std::vector<int> dyn((size_t)needed);
            std::vector<Vec3> f((size_t)needed), t((size_t)needed);
            for (int k = 0; k < needed && k < model_.num_bodies(); ++k) {
                const Transform& tr = state_.transforms[(size_t)k];
                pos[3 * k] = tr.position.x;
                pos[3 * k + 1] = tr.position.y;
                pos[3 * k + 2] = tr.position.z;
                quat[4 * k] = tr.rotation.w;
                quat[4 * k + 1] = tr.rotation.x;
                quat[4 * k + 2] = tr.rotation.y;
                quat[4 * k + 3] = tr.rotation.z;
                dyn[(size_t)k] = model_.bodies[(size_t)k].is_static() ? 0 : 1;
                f[(size_t)k] = state_.forces[(size_t)k];
                t[(size_t)k] = state_.torques[(size_t)k];
            }
            if (!boundary_.empty() && needed > 0) {
                check_pbf(pbf_scene_set_bodies(scene_, needed, pos.data(), quat.data(),
                                               dyn.data()));
                if (pbf_.boundary_two_way && pbf_.boundary_friction != 0.0f) {
                    std::vector<float> lin(3 * (size_t)needed, 0.0f), ang(3 * (size_t)needed, 0.0f);
                    for (int k = 0; k < needed && k < model_.num_bodies(); ++k) {
                        const Vec3& l = state_.linear_velocities[(size_t)k];
                        const Vec3& a = state_.angular_velocities[(size_t)k];
                        lin[3 * k] = l.x;
                        lin[3 * k + 1] = l.y;
                        lin[3 * k + 2] = l.z;
                        ang[3 * k] = a.x;
                        ang[3 * k + 1] = a.y;
                        ang[3 * k + 2] = a.z;
                    }
                    check_pbf(pbf_scene_set_body_velocities(scene_, needed, lin.data(), ang.data()));
                }
            }
            float* fp = needed ? &f[0].x : nullptr;
            float* tp = needed ? &t[0].x : nullptr;
            if (!monitor_.enabled || pbf_.boundary_two_way) {
                // (A two-way step runs only as the whole coupled step.)
                Scope p(monitor_, "fluid.pbf.total");
                check_pbf(pbf_scene_step_coupled(scene_, dt, fp, tp));
            } else {
                // Profiled: the same step (a plain launch sequence instead of
                // the graph) with the device time of every reference phase.
                float ph[PBF_NUM_PHASES];
                {
                    Scope p(monitor_, "fluid.pbf.total");
                    check_pbf(pbf_scene_step_profiled(scene_, dt, ph, nullptr));
                    double at = monitor_.now_us(p.t0);
                    for (int k = 0; k < PBF_NUM_PHASES; ++k) {
                        monitor_.record_device_phase(pbf_phase_name(k), ph[k], at);
                        at += ph[k] * 1e3;
                    }
                }
                if (!boundary_.empty()) {
                    float cp[3];
                    const PerformanceMonitor::Clock::time_point c0 = PerformanceMonitor::Clock::now();
                    check_pbf(pbf_scene_couple_profiled(scene_, dt, fp, tp, cp));
                    const char* names[3] = {"fluid.boundary.positions", "fluid.boundary_density",
                                            "fluid.coupling.total"};
                    double at = monitor_.now_us(c0);
                    for (int k = 0; k < 3; ++k) {
                        monitor_.record_device_phase(names[k], cp[k], at);
                        at += cp[k] * 1e3;
                    }
                }
            }
            for (int k = 0; k < needed && k < model_.num_bodies(); ++k) {
                // With sleep on, a sleeping body that took coupling force
                // wakes (World::apply_force); the test is on the body's
                // summed force and torque changing.
                const Vec3& f0 = state_.forces[(size_t)k];
                const Vec3& t0 = state_.torques[(size_t)k];
                const bool touched = f0.x != f[(size_t)k].x || f0.y != f[(size_t)k].y ||
                                     f0.z != f[(size_t)k].z || t0.x != t[(size_t)k].x ||
                                     t0.y != t[(size_t)k].y || t0.z != t[(size_t)k].z;
                if (touched && solver_.settings().sleep_enabled && state_.is_sleeping(k))
                    state_.wake_body(k);
                state_.forces[(size_t)k] = f[(size_t)k];
                state_.torques[(size_t)k] = t[(size_t)k];
            }
            host_dirty_ = true;
            for (auto& pf : pinned_) pf.stale = true;
        }
        {
            Scope r(monitor_, "fluid.rigid_step");
            step_rigid_pipeline(dt);
        }
        monitor_.record_metric("fluid_particles", (double)n_);
        monitor_.record_metric("boundary_particles", (double)boundary_.size());
        monitor_.record_metric("pbf_solver_iterations", (double)pbf_.solver_iterations);
        monitor_.record_metric("kernel_radius", (double)pbf_.kernel_radius);
    }
    monitor_.end_frame();
}

}  // namespace novaphy_gb300
