// Rigid contacts of the host World: shape boxes, the broad phase, the narrow
// phase, contact islands with sleep, and the sequential-impulse solver.  The
// float operations and their order follow the reference pipeline
// (src/collision/broadphase.cpp, src/collision/narrowphase.cpp,
// src/dynamics/free_body_solver.cpp, src/sim/state.cpp) so that a World
// stepped here matches the reference's bit for bit; the code is this
// library's own.  Compiled with -ffp-contract=off.
#include <algorithm>
#include <limits>

#include "novaphy_host.hpp"

namespace novaphy_gb300 {

namespace {

Vec3 mat_vec(const Mat3& m, const Vec3& v) {
    return {m[0] * v.x + (m[1] * v.y + m[2] * v.z), m[3] * v.x + (m[4] * v.y + m[5] * v.z),
            m[6] * v.x + (m[7] * v.y + m[8] * v.z)};
}

Mat3 mat_mul(const Mat3& a, const Mat3& b) {
    Mat3 c{};
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 3; ++k)
            c[3 * r + k] = a[3 * r] * b[k] + (a[3 * r + 1] * b[3 + k] + a[3 * r + 2] * b[6 + k]);
    return c;
}

Mat3 transposed(const Mat3& m) { return {m[0], m[3], m[6], m[1], m[4], m[7], m[2], m[5], m[8]}; }

Vec3 column(const Mat3& m, int c) { return {m[c], m[3 + c], m[6 + c]}; }

float clampf(float v, float lo, float hi) { return std::max(lo, std::min(v, hi)); }

// Corner k of a box with half extents h: bit 0 picks +x, bit 1 +y, bit 2 +z.
Vec3 corner(const Vec3& h, int k) {
    return {(k & 1) ? h.x : -h.x, (k & 2) ? h.y : -h.y, (k & 4) ? h.z : -h.z};
}

ContactPoint make_contact(const Vec3& normal, float pen, const Vec3& pos, int body_a, int body_b,
                          const CollisionShape& s0, const CollisionShape& s1) {
    ContactPoint c;
    c.normal = normal;
    c.penetration = pen;
    c.position = pos;
    c.body_a = body_a;
    c.body_b = body_b;
    c.friction = combine_friction(s0.friction, s1.friction);
    c.restitution = combine_restitution(s0.restitution, s1.restitution);
    return c;
}

// ---- narrow phase (src/collision/narrowphase.cpp) ----

bool spheres(const CollisionShape& a, const Transform& ta, const CollisionShape& b,
             const Transform& tb, std::vector<ContactPoint>& out) {
    const Vec3 ca = ta.transform_point(a.local_transform.position);
    const Vec3 cb = tb.transform_point(b.local_transform.position);
    const Vec3 diff = cb - ca;
    const float d2 = diff.squaredNorm();
    const float rsum = a.radius + b.radius;
    if (d2 > rsum * rsum) return false;
    const float dist = std::sqrt(d2);
    const Vec3 n = dist < 1e-6f ? Vec3(0.0f, 1.0f, 0.0f) : diff / dist;
    const float pen = rsum - dist;
    out.push_back(make_contact(n, pen, ca + n * (a.radius - pen * 0.5f), a.body_index, b.body_index,
                               a, b));
    return true;
}

// Plane first in the contact (body_a), normal = the plane's.
bool sphere_plane(const CollisionShape& s, const Transform& ts, const CollisionShape& p,
                  std::vector<ContactPoint>& out) {
    const Vec3 c = ts.transform_point(s.local_transform.position);
    const float dist = p.normal.dot(c) - p.offset;
    if (dist > s.radius) return false;
    out.push_back(make_contact(p.normal, s.radius - dist, c - p.normal * dist, p.body_index,
                               s.body_index, s, p));
    return true;
}

// Box first (body_a); the normal points from the box toward the sphere.
bool box_sphere(const CollisionShape& bx, const Transform& tb, const CollisionShape& s,
                const Transform& ts, std::vector<ContactPoint>& out) {
    const Transform box = tb * bx.local_transform;
    const Vec3 centre = ts.transform_point(s.local_transform.position);
    const Vec3 local = box.inverse().transform_point(centre);
    const Vec3& h = bx.half_extents;
    const Vec3 closest(clampf(local.x, -h.x, h.x), clampf(local.y, -h.y, h.y),
                       clampf(local.z, -h.z, h.z));
    const float d2 = (local - closest).squaredNorm();
    if (d2 > s.radius * s.radius) return false;
    const Vec3 wclosest = box.transform_point(closest);
    const float dist = std::sqrt(d2);
    Vec3 n;
    if (dist < 1e-6f) {
        // centre inside the box: push out through the nearest face
        const Vec3 face(h.x - std::abs(local.x), h.y - std::abs(local.y), h.z - std::abs(local.z));
        int axis = 0;
        if (face.y < face[axis]) axis = 1;
        if (face.z < face[axis]) axis = 2;
        Vec3 ln;
        ln[axis] = local[axis] > 0 ? 1.0f : -1.0f;
        n = box.transform_vector(ln);
    } else {
        n = (centre - wclosest) / dist;
    }
    out.push_back(make_contact(n, s.radius - dist, wclosest, bx.body_index, s.body_index, bx, s));
    return true;
}

// One contact per box corner below the plane; plane first (body_a).
bool box_plane(const CollisionShape& bx, const Transform& tb, const CollisionShape& p,
               std::vector<ContactPoint>& out) {
    const Transform box = tb * bx.local_transform;
    bool hit = false;
    for (int k = 0; k < 8; ++k) {
        const Vec3 w = box.transform_point(corner(bx.half_extents, k));
        const float dist = p.normal.dot(w) - p.offset;
        if (dist < 0.0f) {
            out.push_back(make_contact(p.normal, -dist, w - p.normal * dist, p.body_index,
                                       bx.body_index, bx, p));
            hit = true;
        }
    }
    return hit;
}

// Separating-axis test over the 3 + 3 face normals and the 9 edge crosses
// (an edge axis must beat the best face axis by 1e-4 to be kept).  A face
// axis yields the incident box's corners that lie within the reference box
// (0.01 slack), at most 4, shifted half the depth along the normal; with
// none (nor any earlier contact in `out`), or for an edge axis, one contact
// at the midpoint of the centres.
bool box_box(const CollisionShape& a, const Transform& ta, const CollisionShape& b,
             const Transform& tb, std::vector<ContactPoint>& out) {
    const Transform wa = ta * a.local_transform, wb = tb * b.local_transform;
    const Vec3 &ha = a.half_extents, &hb = b.half_extents;
    const Mat3 ra = wa.rotation_matrix(), rb = wb.rotation_matrix();
    const Vec3 d = wb.position - wa.position;
    const Vec3 ax_a[3] = {column(ra, 0), column(ra, 1), column(ra, 2)};
    const Vec3 ax_b[3] = {column(rb, 0), column(rb, 1), column(rb, 2)};
    const Mat3 rat = transposed(ra);
    const Mat3 r = mat_mul(rat, rb);  // B's axes in A's frame
    Mat3 ar;
    for (int k = 0; k < 9; ++k) ar[k] = std::abs(r[k]) + 1e-6f;
    const Vec3 t = mat_vec(rat, d);

    float best = std::numeric_limits<float>::max();
    Vec3 axis_best;
    int best_idx = -1;
    for (int i = 0; i < 3; ++i) {
        const float proj_b = hb.x * ar[3 * i] + hb.y * ar[3 * i + 1] + hb.z * ar[3 * i + 2];
        const float pen = (ha[i] + proj_b) - std::abs(t[i]);
        if (pen < 0) return false;
        if (pen < best) {
            best = pen;
            axis_best = t[i] < 0 ? -ax_a[i] : ax_a[i];
            best_idx = i;
        }
    }
    for (int i = 0; i < 3; ++i) {
        const float proj_a = ha.x * ar[i] + ha.y * ar[3 + i] + ha.z * ar[6 + i];
        const float s = column(r, i).dot(t);
        const float pen = (proj_a + hb[i]) - std::abs(s);
        if (pen < 0) return false;
        if (pen < best) {
            best = pen;
            axis_best = s < 0 ? -ax_b[i] : ax_b[i];
            best_idx = 3 + i;
        }
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            Vec3 axis = ax_a[i].cross(ax_b[j]);
            const float len = axis.norm();
            if (len < 1e-6f) continue;
            axis = axis / len;
            float proj_a = 0, proj_b = 0;
            for (int k = 0; k < 3; ++k) {
                proj_a += ha[k] * std::abs(axis.dot(ax_a[k]));
                proj_b += hb[k] * std::abs(axis.dot(ax_b[k]));
            }
            const float s = axis.dot(d);
            const float pen = (proj_a + proj_b) - std::abs(s);
            if (pen < 0) return false;
            if (pen < best - 1e-4f) {
                best = pen;
                axis_best = s < 0 ? -axis : axis;
                best_idx = 6 + 3 * i + j;
            }
        }

    const Vec3 mid = wa.position + d * 0.5f;
    if (best_idx < 6) {
        const bool a_ref = best_idx < 3;
        const Vec3& ref_h = a_ref ? ha : hb;
        const Vec3& inc_h = a_ref ? hb : ha;
        const Transform& ref = a_ref ? wa : wb;
        const Transform& inc = a_ref ? wb : wa;
        const float pen = std::max(0.0f, best);
        int found = 0;
        for (int k = 0; k < 8 && found < 4; ++k) {
            const Vec3 w = inc.transform_point(corner(inc_h, k));
            const Vec3 l = ref.inverse().transform_point(w);
            if (std::abs(l.x) <= ref_h.x + 0.01f && std::abs(l.y) <= ref_h.y + 0.01f &&
                std::abs(l.z) <= ref_h.z + 0.01f) {
                const float off = 0.5f * pen;
                const Vec3 pos = a_ref ? w + axis_best * off : w - axis_best * off;
                out.push_back(make_contact(axis_best, pen, pos, a.body_index, b.body_index, a, b));
                ++found;
            }
        }
        if (out.empty())
            out.push_back(make_contact(axis_best, best, mid, a.body_index, b.body_index, a, b));
    } else {
        out.push_back(make_contact(axis_best, best, mid, a.body_index, b.body_index, a, b));
    }
    return !out.empty();
}

}  // namespace

void AABB::expand(const Vec3& p) {
    min = Vec3(std::min(min.x, p.x), std::min(min.y, p.y), std::min(min.z, p.z));
    max = Vec3(std::max(max.x, p.x), std::max(max.y, p.y), std::max(max.z, p.z));
}

AABB CollisionShape::compute_aabb(const Transform& body_transform) const {
    const Transform w = body_transform * local_transform;
    switch (type) {
        case ShapeType::Box: {
            AABB box;
            for (int k = 0; k < 8; ++k) box.expand(w.transform_point(corner(half_extents, k)));
            return box;
        }
        case ShapeType::Sphere:
            return AABB::from_sphere(w.position, radius);
        case ShapeType::Plane:
            return AABB(Vec3(-1e6f, -1e6f, -1e6f), Vec3(1e6f, 1e6f, 1e6f));
    }
    return AABB();
}

bool collide_shapes(const CollisionShape& a, const Transform& ta, const CollisionShape& b,
                    const Transform& tb, std::vector<ContactPoint>& contacts) {
    using S = ShapeType;
    if (a.type == S::Sphere && b.type == S::Sphere) return spheres(a, ta, b, tb, contacts);
    if (a.type == S::Sphere && b.type == S::Plane) return sphere_plane(a, ta, b, contacts);
    if (a.type == S::Plane && b.type == S::Sphere) return sphere_plane(b, tb, a, contacts);
    if (a.type == S::Box && b.type == S::Sphere) return box_sphere(a, ta, b, tb, contacts);
    if (a.type == S::Sphere && b.type == S::Box) {
        // box-sphere with the roles swapped back: every contact in the list
        // is turned around, as the reference dispatcher does
        const bool hit = box_sphere(b, tb, a, ta, contacts);
        for (ContactPoint& c : contacts) {
            c.normal = -c.normal;
            std::swap(c.body_a, c.body_b);
        }
        return hit;
    }
    if (a.type == S::Box && b.type == S::Plane) return box_plane(a, ta, b, contacts);
    if (a.type == S::Plane && b.type == S::Box) return box_plane(b, tb, a, contacts);
    if (a.type == S::Box && b.type == S::Box) return box_box(a, ta, b, tb, contacts);
    return false;
}

// ---- broad phase ----

void SweepAndPrune::update(const std::vector<AABB>& aabbs, const std::vector<bool>& static_mask) {
    const int n = (int)aabbs.size();
    if ((int)static_mask.size() < n) throw std::invalid_argument("static_mask shorter than aabbs");
    // Sweep over x in order of the lower bound: a box meets every later box
    // whose lower bound is <= its upper bound; y and z decide the rest.
    order_.resize((size_t)n);
    for (int i = 0; i < n; ++i) order_[(size_t)i] = i;
    std::sort(order_.begin(), order_.end(), [&](int p, int q) {
        const float a = aabbs[(size_t)p].min.x, b = aabbs[(size_t)q].min.x;
        return a < b || (!(b < a) && p < q);
    });
    pairs_.clear();
    for (int i = 0; i < n; ++i) {
        const int a = order_[(size_t)i];
        const AABB& A = aabbs[(size_t)a];
        for (int j = i + 1; j < n; ++j) {
            const int b = order_[(size_t)j];
            const AABB& B = aabbs[(size_t)b];
            if (B.min.x > A.max.x) break;
            if (static_mask[(size_t)a] && static_mask[(size_t)b]) continue;
            if (A.min.y <= B.max.y && A.max.y >= B.min.y && A.min.z <= B.max.z &&
                A.max.z >= B.min.z)
                pairs_.push_back({std::min(a, b), std::max(a, b)});
        }
    }
    std::sort(pairs_.begin(), pairs_.end(), [](const BroadPhasePair& p, const BroadPhasePair& q) {
        return p.body_a < q.body_a || (p.body_a == q.body_a && p.body_b < q.body_b);
    });
    pairs_.erase(std::unique(pairs_.begin(), pairs_.end()), pairs_.end());
}

// ---- state and sleep (src/sim/state.cpp) ----

void SimState::init(const std::vector<Transform>& t) {
    const size_t n = t.size();
    transforms = t;
    linear_velocities.assign(n, Vec3{});
    angular_velocities.assign(n, Vec3{});
    forces.assign(n, Vec3{});
    torques.assign(n, Vec3{});
    sleeping.assign(n, 0);
    sleep_timer.assign(n, 0.0f);
    smoothed_energy.assign(n, 0.0f);
    island_id.assign(n, -1);
}

void SimState::clear_forces() {
    for (Vec3& f : forces) f = Vec3{};
    for (Vec3& t : torques) t = Vec3{};
}

void SimState::set_linear_velocity(int i, const Vec3& v) {
    if (i >= 0 && i < (int)linear_velocities.size()) linear_velocities[(size_t)i] = v;
}

void SimState::set_angular_velocity(int i, const Vec3& w) {
    if (i >= 0 && i < (int)angular_velocities.size()) angular_velocities[(size_t)i] = w;
}

void SimState::apply_force(int i, const Vec3& f) {
    if (i >= 0 && i < (int)forces.size()) forces[(size_t)i] += f;
}

void SimState::apply_torque(int i, const Vec3& t) {
    if (i >= 0 && i < (int)torques.size()) torques[(size_t)i] += t;
}

// A woken body starts from rest with a small energy so that it does not fall
// asleep again at once; its island wakes with it.
void SimState::wake_body(int i) {
    if (i < 0 || i >= (int)sleeping.size()) return;
    sleeping[(size_t)i] = 0;
    sleep_timer[(size_t)i] = 0.0f;
    smoothed_energy[(size_t)i] = 0.02f;
    linear_velocities[(size_t)i] = Vec3{};
    angular_velocities[(size_t)i] = Vec3{};
    propagate_wake_through_island(i);
}

bool SimState::is_sleeping(int i) const {
    return i >= 0 && i < (int)sleeping.size() && sleeping[(size_t)i] != 0;
}

void SimState::update_energy(int i, float energy, float alpha) {
    if (i >= 0 && i < (int)smoothed_energy.size())
        smoothed_energy[(size_t)i] = alpha * smoothed_energy[(size_t)i] + (1.0f - alpha) * energy;
}

float SimState::get_smoothed_energy(int i) const {
    return (i >= 0 && i < (int)smoothed_energy.size()) ? smoothed_energy[(size_t)i] : 0.0f;
}

// Islands are the connected components of the contact graph over all bodies
// (static ones included; world-owned shapes join nothing), numbered in order
// of their lowest body index.
void SimState::build_islands(const std::vector<ContactPoint>& contacts) {
    const int n = (int)sleeping.size();
    std::vector<int> parent((size_t)n), rank((size_t)n, 0);
    for (int i = 0; i < n; ++i) parent[(size_t)i] = i;
    auto root = [&](int x) {
        int r = x;
        while (parent[(size_t)r] != r) r = parent[(size_t)r];
        while (parent[(size_t)x] != r) {
            const int next = parent[(size_t)x];
            parent[(size_t)x] = r;
            x = next;
        }
        return r;
    };
    for (const ContactPoint& c : contacts) {
        if (c.body_a < 0 || c.body_b < 0 || c.body_a >= n || c.body_b >= n) continue;
        const int x = root(c.body_a), y = root(c.body_b);
        if (x == y) continue;
        if (rank[(size_t)x] < rank[(size_t)y]) {
            parent[(size_t)x] = y;
        } else {
            parent[(size_t)y] = x;
            if (rank[(size_t)x] == rank[(size_t)y]) ++rank[(size_t)x];
        }
    }
    island_id.assign((size_t)n, -1);
    int next = 0;
    for (int i = 0; i < n; ++i) {
        const int r = root(i);
        if (island_id[(size_t)r] < 0) island_id[(size_t)r] = next++;
        island_id[(size_t)i] = island_id[(size_t)r];
    }
}

// Timers grow by dt while the smoothed energy is under the threshold and
// reset otherwise; an island sleeps when no member is above the threshold
// and every member's timer reached time_threshold.  Sleeping bodies are
// brought to rest; bodies outside any island stay awake.
void SimState::evaluate_sleep(float dt, float energy_threshold, float time_threshold) {
    const int n = (int)sleeping.size();
    int islands = 0;
    for (int i = 0; i < n; ++i) islands = std::max(islands, island_id[(size_t)i] + 1);
    // per island: some member above the energy threshold / every member's
    // timer at least time_threshold (one pass each instead of a scan per body)
    std::vector<char> awake((size_t)islands, 0), timed((size_t)islands, 1);
    for (int i = 0; i < n; ++i) {
        const int isl = island_id[(size_t)i];
        if (isl < 0) continue;
        if (smoothed_energy[(size_t)i] < energy_threshold) {
            sleep_timer[(size_t)i] += dt;
        } else {
            sleep_timer[(size_t)i] = 0.0f;
            awake[(size_t)isl] = 1;
        }
    }
    for (int i = 0; i < n; ++i) {
        const int isl = island_id[(size_t)i];
        if (isl >= 0 && sleep_timer[(size_t)i] < time_threshold) timed[(size_t)isl] = 0;
    }
    for (int i = 0; i < n; ++i) {
        const int isl = island_id[(size_t)i];
        if (isl >= 0 && !awake[(size_t)isl] && timed[(size_t)isl]) {
            sleeping[(size_t)i] = 1;
            linear_velocities[(size_t)i] = Vec3{};
            angular_velocities[(size_t)i] = Vec3{};
        } else {
            sleeping[(size_t)i] = 0;
        }
    }
}

void SimState::propagate_wake_through_island(int i) {
    if (i < 0 || i >= (int)island_id.size()) return;
    const int isl = island_id[(size_t)i];
    if (isl < 0) return;
    for (size_t k = 0; k < island_id.size(); ++k)
        if (island_id[k] == isl && sleeping[k] != 0) {
            sleeping[k] = 0;
            sleep_timer[k] = 0.0f;
            smoothed_energy[k] = 0.02f;
        }
}

// ---- contact solver (src/dynamics/free_body_solver.cpp) ----

namespace {

// Records the time from construction to destruction as a monitor phase.
struct Phase {
    PerformanceMonitor* m;
    const char* name;
    PerformanceMonitor::Clock::time_point t0 = PerformanceMonitor::Clock::now();
    Phase(PerformanceMonitor* mon, const char* n) : m(mon), name(n) {}
    ~Phase() {
        if (m)
            m->record_phase(name,
                            std::chrono::duration<double, std::milli>(
                                PerformanceMonitor::Clock::now() - t0)
                                .count(),
                            t0);
    }
};

bool moves(const std::vector<RigidBody>& bodies, int b) {
    return b >= 0 && !bodies[(size_t)b].is_static();
}

Vec3 point_velocity(const std::vector<Vec3>& lin, const std::vector<Vec3>& ang, int b,
                    const Vec3& r) {
    return b >= 0 ? lin[(size_t)b] + ang[(size_t)b].cross(r) : Vec3{};
}

}  // namespace

void ContactSolver::solve(std::vector<ContactPoint>& contacts, const std::vector<RigidBody>& bodies,
                          const std::vector<Transform>& transforms, std::vector<Vec3>& lin,
                          std::vector<Vec3>& ang, const std::vector<int>& sleeping, float dt,
                          PerformanceMonitor* monitor) {
    if (contacts.empty()) return;
    {
        Phase ph(monitor, "world.solver.pre_step");
        prepare(contacts, bodies, transforms, lin, ang, sleeping, dt);
    }
    if (settings_.warm_starting) {
        Phase ph(monitor, "world.solver.warm_start");
        for (size_t i = 0; i < contacts.size(); ++i) {
            const ContactPoint& c = contacts[i];
            const Row& w = rows_[i];
            if (w.k_n == 0.0f) continue;  // both bodies asleep
            const Vec3 p = c.normal * c.accumulated_normal_impulse +
                           w.t1 * c.accumulated_tangent_impulse_1 +
                           w.t2 * c.accumulated_tangent_impulse_2;
            if (moves(bodies, c.body_a)) {
                lin[(size_t)c.body_a] -= p * bodies[(size_t)c.body_a].inv_mass();
                ang[(size_t)c.body_a] -= mat_vec(w.inv_i_a, w.r_a.cross(p));
            }
            if (moves(bodies, c.body_b)) {
                lin[(size_t)c.body_b] += p * bodies[(size_t)c.body_b].inv_mass();
                ang[(size_t)c.body_b] += mat_vec(w.inv_i_b, w.r_b.cross(p));
            }
        }
    }
    for (int it = 0; it < settings_.velocity_iterations; ++it) {
        Phase ph(monitor, "world.solver.iteration.solve_velocity");
        sweep(contacts, bodies, lin, ang);
    }
}

void ContactSolver::prepare(std::vector<ContactPoint>& contacts,
                            const std::vector<RigidBody>& bodies,
                            const std::vector<Transform>& transforms, const std::vector<Vec3>& lin,
                            const std::vector<Vec3>& ang, const std::vector<int>& sleeping,
                            float dt) {
    rows_.resize(contacts.size());
    const int ns = (int)sleeping.size();
    auto asleep = [&](int b) { return b >= 0 && b < ns && sleeping[(size_t)b] != 0; };
    // inverse of 1/m + 1/m' + (r x u).(I^-1 (r x u)) + (r' x u).(I'^-1 (r' x u))
    auto eff_mass = [](float ima, float imb, const Row& w, const Vec3& u) {
        const Vec3 ra = w.r_a.cross(u), rb = w.r_b.cross(u);
        float k = ima + imb + ra.dot(mat_vec(w.inv_i_a, ra)) + rb.dot(mat_vec(w.inv_i_b, rb));
        if (k > 0) k = 1.0f / k;
        return k;
    };
    for (size_t i = 0; i < contacts.size(); ++i) {
        ContactPoint& c = contacts[i];
        Row& w = rows_[i];
        if (asleep(c.body_a) && asleep(c.body_b)) {
            w.k_n = w.k_t1 = w.k_t2 = 0.0f;
            continue;
        }
        w.r_a = c.body_a >= 0 ? c.position - transforms[(size_t)c.body_a].position : Vec3{};
        w.r_b = c.body_b >= 0 ? c.position - transforms[(size_t)c.body_b].position : Vec3{};
        const float ima = c.body_a >= 0 ? bodies[(size_t)c.body_a].inv_mass() : 0.0f;
        const float imb = c.body_b >= 0 ? bodies[(size_t)c.body_b].inv_mass() : 0.0f;
        // world inverse inertia R I^-1 R^T
        auto world_inv = [&](int b) {
            if (!moves(bodies, b)) return Mat3{};
            const Mat3 r = transforms[(size_t)b].rotation_matrix();
            return mat_mul(mat_mul(r, bodies[(size_t)b].inv_inertia()), transposed(r));
        };
        w.inv_i_a = world_inv(c.body_a);
        w.inv_i_b = world_inv(c.body_b);
        w.k_n = eff_mass(ima, imb, w, c.normal);
        w.t1 = (std::abs(c.normal.x) < 0.9f ? c.normal.cross(Vec3(1, 0, 0))
                                            : c.normal.cross(Vec3(0, 1, 0)))
                   .normalized();
        w.t2 = c.normal.cross(w.t1);
        w.k_t1 = eff_mass(ima, imb, w, w.t1);
        w.k_t2 = eff_mass(ima, imb, w, w.t2);
        // Baumgarte push-out beyond the slop, plus restitution on fast approach
        const float depth = std::max(0.0f, c.penetration - settings_.slop);
        w.bias = settings_.baumgarte * depth / dt;
        const Vec3 va = point_velocity(lin, ang, c.body_a, w.r_a);
        const Vec3 vb = point_velocity(lin, ang, c.body_b, w.r_b);
        const float vn = c.normal.dot(vb - va);
        if (vn < -1.0f) w.bias += c.restitution * vn;
        if (!settings_.warm_starting) {
            c.accumulated_normal_impulse = 0.0f;
            c.accumulated_tangent_impulse_1 = 0.0f;
            c.accumulated_tangent_impulse_2 = 0.0f;
        }
    }
}

void ContactSolver::sweep(std::vector<ContactPoint>& contacts, const std::vector<RigidBody>& bodies,
                          std::vector<Vec3>& lin, std::vector<Vec3>& ang) {
    for (size_t i = 0; i < contacts.size(); ++i) {
        ContactPoint& c = contacts[i];
        const Row& w = rows_[i];
        if (w.k_n == 0.0f) continue;
        const float ima = c.body_a >= 0 ? bodies[(size_t)c.body_a].inv_mass() : 0.0f;
        const float imb = c.body_b >= 0 ? bodies[(size_t)c.body_b].inv_mass() : 0.0f;
        const bool ma = moves(bodies, c.body_a), mb = moves(bodies, c.body_b);
        auto push = [&](const Vec3& p) {
            if (ma) {
                lin[(size_t)c.body_a] -= p * ima;
                ang[(size_t)c.body_a] -= mat_vec(w.inv_i_a, w.r_a.cross(p));
            }
            if (mb) {
                lin[(size_t)c.body_b] += p * imb;
                ang[(size_t)c.body_b] += mat_vec(w.inv_i_b, w.r_b.cross(p));
            }
        };
        auto rel_vel = [&]() {
            const Vec3 va = point_velocity(lin, ang, c.body_a, w.r_a);
            const Vec3 vb = point_velocity(lin, ang, c.body_b, w.r_b);
            return vb - va;
        };
        // normal row: accumulated impulse stays >= 0
        float dn = w.k_n * (-rel_vel().dot(c.normal) + w.bias);
        const float old_n = c.accumulated_normal_impulse;
        c.accumulated_normal_impulse = std::max(0.0f, old_n + dn);
        dn = c.accumulated_normal_impulse - old_n;
        push(c.normal * dn);
        // friction rows, each re-reading the relative velocity, inside
        // |impulse| <= friction * normal impulse
        const float cap = c.friction * c.accumulated_normal_impulse;
        float d1 = w.k_t1 * -rel_vel().dot(w.t1);
        const float old_1 = c.accumulated_tangent_impulse_1;
        c.accumulated_tangent_impulse_1 = std::max(-cap, std::min(cap, old_1 + d1));
        d1 = c.accumulated_tangent_impulse_1 - old_1;
        push(w.t1 * d1);
        float d2 = w.k_t2 * -rel_vel().dot(w.t2);
        const float old_2 = c.accumulated_tangent_impulse_2;
        c.accumulated_tangent_impulse_2 = std::max(-cap, std::min(cap, old_2 + d2));
        d2 = c.accumulated_tangent_impulse_2 - old_2;
        push(w.t2 * d2);
    }
}

}  // namespace novaphy_gb300
