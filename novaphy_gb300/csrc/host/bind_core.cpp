// pybind11 module novaphy_gb300._core: NovaPhy's fluid bindings
// (python/bindings/bind_fluid.cpp) with the same class, method and argument
// names, plus the slices of the sim/core/math bindings that FluidWorld and its
// callers use (bind_sim.cpp, bind_core.cpp, bind_math.cpp,
// bind_performance.cpp).  Vector3 values are float32 numpy arrays of shape
// (3,), like the reference's Eigen binding; any length-3 sequence is accepted.
#include <cstdint>
#include <cstring>

#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include "novaphy_host.hpp"

namespace py = pybind11;
using namespace novaphy_gb300;

namespace pybind11 {
namespace detail {
template <>
struct type_caster<Vec3> {
    PYBIND11_TYPE_CASTER(Vec3, const_name("Vector3"));
    bool load(handle src, bool) {
        if (!src || !PySequence_Check(src.ptr()) || PyUnicode_Check(src.ptr())) return false;
        auto seq = reinterpret_borrow<sequence>(src);
        if (seq.size() != 3) return false;
        try {
            for (size_t i = 0; i < 3; ++i) value[(int)i] = seq[i].cast<float>();
        } catch (const cast_error&) {
            return false;
        }
        return true;
    }
    static handle cast(const Vec3& v, return_value_policy, handle) {
        array_t<float> a(3);
        auto m = a.mutable_unchecked<1>();
        m(0) = v.x;
        m(1) = v.y;
        m(2) = v.z;
        return a.release();
    }
};
}  // namespace detail
}  // namespace pybind11

namespace {

py::array_t<float> mat3_array(const Mat3& m) {
    py::array_t<float> a({3, 3});
    std::memcpy(a.mutable_data(), m.data(), 9 * sizeof(float));
    return a;
}

py::array_t<float> positions_array(const std::vector<Vec3>& v) {
    py::array_t<float> a({(py::ssize_t)v.size(), (py::ssize_t)3});
    if (!v.empty()) std::memcpy(a.mutable_data(), &v[0].x, v.size() * sizeof(Vec3));
    return a;
}

// A fluid field in device memory, handed to other libraries through
// __cuda_array_interface__ (version 3) without a copy.  Keeps its world alive.
struct DeviceFieldView {
    uintptr_t ptr = 0;
    py::ssize_t n = 0;
    bool vec = false;
    py::object owner;
    py::dict interface() const {
        py::dict d;
        if (vec) {
            d["shape"] = py::make_tuple(n, 3);
            d["strides"] = py::make_tuple(16, 4);  // float4 rows on the device
        } else {
            d["shape"] = py::make_tuple(n);
            d["strides"] = py::make_tuple(4);
        }
        d["typestr"] = "<f4";
        d["data"] = py::make_tuple(n > 0 ? ptr : (uintptr_t)0, false);
        d["version"] = 3;
        return d;
    }
};

const char* const kFieldNames[4] = {"positions", "velocities", "densities", "lambdas"};

}  // namespace

PYBIND11_MODULE(_core, m) {
    m.doc() = "NovaPhy's PBF fluid API on the GB300 (sm_103a) behind a C ABI";

    // --- math / core slices ---
    py::class_<Transform>(m, "Transform")
        .def(py::init<>())
        .def(py::init([](const Vec3& p, py::sequence q) {
                 if (q.size() != 4) throw py::value_error("rotation must be [x, y, z, w]");
                 return Transform(p, Quat{q[3].cast<float>(), q[0].cast<float>(),
                                          q[1].cast<float>(), q[2].cast<float>()});
             }),
             py::arg("position"), py::arg("rotation"))
        .def_readwrite("position", &Transform::position)
        .def_property(
            "rotation",
            [](const Transform& t) {
                py::array_t<float> a(4);
                auto r = a.mutable_unchecked<1>();
                r(0) = t.rotation.x;
                r(1) = t.rotation.y;
                r(2) = t.rotation.z;
                r(3) = t.rotation.w;
                return a;
            },
            [](Transform& t, py::sequence q) {
                t.rotation = Quat{q[3].cast<float>(), q[0].cast<float>(), q[1].cast<float>(),
                                  q[2].cast<float>()};
            })
        .def("transform_point", &Transform::transform_point, py::arg("point"))
        .def("transform_vector", &Transform::transform_vector, py::arg("vector"))
        .def("inverse", &Transform::inverse)
        .def("rotation_matrix", [](const Transform& t) { return mat3_array(t.rotation_matrix()); })
        .def("__mul__", &Transform::operator*, py::arg("other"))
        .def("__repr__",
             [](const Transform& t) {
                 return "Transform(pos=[" + std::to_string(t.position.x) + ", " +
                        std::to_string(t.position.y) + ", " + std::to_string(t.position.z) +
                        "], rot=[" + std::to_string(t.rotation.w) + ", " +
                        std::to_string(t.rotation.x) + ", " + std::to_string(t.rotation.y) +
                        ", " + std::to_string(t.rotation.z) + "])";
             })
        .def_static("identity", &Transform::identity)
        .def_static(
            "from_rotation",
            [](py::sequence q) {
                if (q.size() != 4) throw py::value_error("rotation must be [x, y, z, w]");
                return Transform(Vec3{}, Quat{q[3].cast<float>(), q[0].cast<float>(),
                                              q[1].cast<float>(), q[2].cast<float>()});
            },
            py::arg("q"))
        .def_static("from_translation", &Transform::from_translation, py::arg("translation"))
        .def_static("from_axis_angle", &Transform::from_axis_angle, py::arg("axis"),
                    py::arg("angle"));

    // math_utils.h helpers: [v]x with skew(a) b = a x b, and angle conversions
    m.def(
        "skew",
        [](const Vec3& v) {
            return mat3_array(Mat3{0.0f, -v.z, v.y, v.z, 0.0f, -v.x, -v.y, v.x, 0.0f});
        },
        py::arg("v"));
    m.def("deg2rad", [](float deg) { return deg * kPi / 180.0f; }, py::arg("deg"));
    m.def("rad2deg", [](float rad) { return rad * 180.0f / kPi; }, py::arg("rad"));

    py::enum_<ShapeType>(m, "ShapeType")
        .value("Box", ShapeType::Box)
        .value("Sphere", ShapeType::Sphere)
        .value("Plane", ShapeType::Plane);

    py::class_<CollisionShape>(m, "CollisionShape")
        .def(py::init<>())
        .def_readwrite("type", &CollisionShape::type)
        .def_readwrite("body_index", &CollisionShape::body_index)
        .def_readwrite("local_transform", &CollisionShape::local_transform)
        .def_readwrite("friction", &CollisionShape::friction)
        .def_readwrite("restitution", &CollisionShape::restitution)
        .def_readwrite("box_half_extents", &CollisionShape::half_extents)
        .def_readwrite("sphere_radius", &CollisionShape::radius)
        .def_readwrite("plane_normal", &CollisionShape::normal)
        .def_readwrite("plane_offset", &CollisionShape::offset)
        .def_static("make_box", &CollisionShape::make_box, py::arg("half_extents"),
                    py::arg("body_idx"), py::arg("local") = Transform::identity(),
                    py::arg("friction") = 0.5f, py::arg("restitution") = 0.3f)
        .def_static("make_sphere", &CollisionShape::make_sphere, py::arg("radius"),
                    py::arg("body_idx"), py::arg("local") = Transform::identity(),
                    py::arg("friction") = 0.5f, py::arg("restitution") = 0.3f)
        .def_static("make_plane", &CollisionShape::make_plane, py::arg("normal"), py::arg("offset"),
                    py::arg("friction") = 0.5f, py::arg("restitution") = 0.0f)
        .def("compute_aabb", &CollisionShape::compute_aabb, py::arg("body_transform"));

    py::class_<AABB>(m, "AABB")
        .def(py::init<>())
        .def(py::init<const Vec3&, const Vec3&>(), py::arg("min"), py::arg("max"))
        .def_readwrite("min", &AABB::min)
        .def_readwrite("max", &AABB::max)
        .def("overlaps", &AABB::overlaps, py::arg("other"))
        .def("center", &AABB::center)
        .def("half_extents", &AABB::half_extents)
        .def("surface_area", &AABB::surface_area)
        .def("is_valid", &AABB::is_valid)
        .def_static("from_sphere", &AABB::from_sphere, py::arg("center"), py::arg("radius"));

    py::class_<ContactPoint>(m, "ContactPoint")
        .def(py::init<>())
        .def_readwrite("position", &ContactPoint::position)
        .def_readwrite("normal", &ContactPoint::normal)
        .def_readwrite("penetration", &ContactPoint::penetration)
        .def_readwrite("body_a", &ContactPoint::body_a)
        .def_readwrite("body_b", &ContactPoint::body_b)
        .def_readwrite("friction", &ContactPoint::friction)
        .def_readwrite("restitution", &ContactPoint::restitution);

    py::class_<BroadPhasePair>(m, "BroadPhasePair")
        .def(py::init<>())
        .def_readwrite("body_a", &BroadPhasePair::body_a)
        .def_readwrite("body_b", &BroadPhasePair::body_b);

    py::class_<SweepAndPrune>(m, "SweepAndPrune")
        .def(py::init<>())
        .def("update", &SweepAndPrune::update, py::arg("aabbs"), py::arg("static_mask"))
        .def("get_pairs", &SweepAndPrune::get_pairs);

    // World vertices of per-instance local vertices: out[i*V + j] =
    // R(quats[b]) local[i, j] + positions[b] with b = body_indices[i]
    // (bind_sim.cpp's batched transform for rendering).  Shapes and indices
    // are checked; the GIL is released for the loop.
    m.def(
        "batch_transform_vertices",
        [](py::array_t<float, py::array::c_style | py::array::forcecast> positions,
           py::array_t<float, py::array::c_style | py::array::forcecast> quats,
           py::array_t<int32_t, py::array::c_style | py::array::forcecast> body_indices,
           py::array_t<float, py::array::c_style | py::array::forcecast> local_verts,
           py::array_t<float, py::array::c_style> out_verts) {
            if (positions.ndim() != 2 || positions.shape(1) != 3 || quats.ndim() != 2 ||
                quats.shape(1) != 4 || quats.shape(0) != positions.shape(0))
                throw py::value_error("positions (B, 3) and quats (B, 4) expected");
            const py::ssize_t nb = positions.shape(0);
            if (body_indices.ndim() != 1 || local_verts.ndim() != 3 || local_verts.shape(2) != 3 ||
                local_verts.shape(0) != body_indices.shape(0))
                throw py::value_error("body_indices (N,) and local_verts (N, V, 3) expected");
            const py::ssize_t n = body_indices.shape(0), nv = local_verts.shape(1);
            if (out_verts.ndim() != 2 || out_verts.shape(1) != 3 || out_verts.shape(0) < n * nv)
                throw py::value_error("out_vertices (N*V, 3) expected");
            const int32_t* idx = body_indices.data();
            for (py::ssize_t i = 0; i < n; ++i)
                if (idx[i] < 0 || idx[i] >= nb) throw py::index_error("body index out of range");
            const float* P = positions.data();
            const float* Q = quats.data();
            const float* L = local_verts.data();
            float* O = out_verts.mutable_data();
            py::gil_scoped_release release;
            for (py::ssize_t i = 0; i < n; ++i) {
                const py::ssize_t b = idx[i];
                const Quat q{Q[4 * b + 3], Q[4 * b], Q[4 * b + 1], Q[4 * b + 2]};
                const Mat3 r = q.rotation_matrix();
                const Vec3 p(P[3 * b], P[3 * b + 1], P[3 * b + 2]);
                for (py::ssize_t j = 0; j < nv; ++j) {
                    const float* v = L + 3 * (i * nv + j);
                    float* o = O + 3 * (i * nv + j);
                    o[0] = r[0] * v[0] + r[1] * v[1] + r[2] * v[2] + p.x;
                    o[1] = r[3] * v[0] + r[4] * v[1] + r[5] * v[2] + p.y;
                    o[2] = r[6] * v[0] + r[7] * v[1] + r[8] * v[2] + p.z;
                }
            }
        },
        py::arg("positions"), py::arg("quats"), py::arg("body_indices"), py::arg("local_verts"),
        py::arg("out_vertices"));

    m.def(
        "collide_shapes",
        [](const CollisionShape& a, const Transform& ta, const CollisionShape& b,
           const Transform& tb) {
            std::vector<ContactPoint> c;
            const bool hit = collide_shapes(a, ta, b, tb, c);
            return py::make_tuple(hit, c);
        },
        py::arg("shape_a"), py::arg("transform_a"), py::arg("shape_b"), py::arg("transform_b"));

    py::class_<RigidBody>(m, "RigidBody")
        .def(py::init<>())
        .def_readwrite("mass", &RigidBody::mass)
        .def_readwrite("com", &RigidBody::com)
        .def("inv_mass", &RigidBody::inv_mass)
        .def("inv_inertia", [](const RigidBody& b) {
            const auto a = b.inv_inertia();
            return std::vector<float>(a.begin(), a.end());
        })
        .def_property(
            "inertia",
            [](const RigidBody& b) {
                py::array_t<float> a({3, 3});
                std::memcpy(a.mutable_data(), b.inertia.data(), 9 * sizeof(float));
                return a;
            },
            [](RigidBody& b, py::array_t<float, py::array::c_style | py::array::forcecast> a) {
                if (a.size() != 9) throw py::value_error("inertia must be 3x3");
                std::memcpy(b.inertia.data(), a.data(), 9 * sizeof(float));
            })
        .def("is_static", &RigidBody::is_static)
        .def_static("from_box", &RigidBody::from_box, py::arg("mass"), py::arg("half_extents"))
        .def_static("from_sphere", &RigidBody::from_sphere, py::arg("mass"), py::arg("radius"))
        .def_static("make_static", &RigidBody::make_static);

    py::class_<Model>(m, "Model")
        .def(py::init<>())
        .def_readonly("bodies", &Model::bodies)
        .def_readonly("shapes", &Model::shapes)
        .def_readonly("initial_transforms", &Model::initial_transforms)
        .def_property_readonly("num_bodies", &Model::num_bodies)
        .def_property_readonly("num_shapes", &Model::num_shapes);

    py::class_<ModelBuilder>(m, "ModelBuilder")
        .def(py::init<>())
        .def("add_body", &ModelBuilder::add_body, py::arg("body"),
             py::arg("transform") = Transform::identity())
        .def("add_shape", &ModelBuilder::add_shape, py::arg("shape"))
        .def("add_ground_plane", &ModelBuilder::add_ground_plane, py::arg("y") = 0.0f,
             py::arg("friction") = 0.5f, py::arg("restitution") = 0.0f)
        .def("build", &ModelBuilder::build)
        .def_property_readonly("num_bodies", &ModelBuilder::num_bodies)
        .def_property_readonly("num_shapes", &ModelBuilder::num_shapes);

    py::class_<SolverSettings>(m, "SolverSettings")
        .def(py::init<>())
        .def_readwrite("velocity_iterations", &SolverSettings::velocity_iterations)
        .def_readwrite("baumgarte", &SolverSettings::baumgarte)
        .def_readwrite("slop", &SolverSettings::slop)
        .def_readwrite("warm_starting", &SolverSettings::warm_starting)
        .def_readwrite("sleep_enabled", &SolverSettings::sleep_enabled)
        .def_readwrite("sleep_energy_threshold", &SolverSettings::sleep_energy_threshold)
        .def_readwrite("sleep_time_required", &SolverSettings::sleep_time_required)
        .def_readwrite("sleep_ema_alpha", &SolverSettings::sleep_ema_alpha);

    py::class_<SimState>(m, "SimState")
        .def(py::init<>())
        .def_readonly("transforms", &SimState::transforms)
        .def_readonly("linear_velocities", &SimState::linear_velocities)
        .def_readonly("angular_velocities", &SimState::angular_velocities)
        .def("set_linear_velocity", &SimState::set_linear_velocity, py::arg("body_index"),
             py::arg("velocity"))
        .def("set_angular_velocity", &SimState::set_angular_velocity, py::arg("body_index"),
             py::arg("velocity"))
        .def("apply_force", &SimState::apply_force, py::arg("body_index"), py::arg("force"))
        .def("apply_torque", &SimState::apply_torque, py::arg("body_index"), py::arg("torque"))
        .def("get_transforms_numpy",
             [](const SimState& s) {
                 // (N, 3) positions and (N, 4) quaternions [x, y, z, w], one call
                 const py::ssize_t n = (py::ssize_t)s.transforms.size();
                 py::array_t<float> pos({n, (py::ssize_t)3}), quat({n, (py::ssize_t)4});
                 float* p = pos.mutable_data();
                 float* q = quat.mutable_data();
                 for (py::ssize_t i = 0; i < n; ++i) {
                     const Transform& t = s.transforms[(size_t)i];
                     p[3 * i] = t.position.x, p[3 * i + 1] = t.position.y, p[3 * i + 2] = t.position.z;
                     q[4 * i] = t.rotation.x, q[4 * i + 1] = t.rotation.y;
                     q[4 * i + 2] = t.rotation.z, q[4 * i + 3] = t.rotation.w;
                 }
                 return py::make_tuple(pos, quat);
             })
        .def("get_transforms_into",
             [](const SimState& s, py::array_t<float, py::array::c_style> pos,
                py::array_t<float, py::array::c_style> quat) {
                 const py::ssize_t n = (py::ssize_t)s.transforms.size();
                 if (pos.ndim() != 2 || pos.shape(0) < n || pos.shape(1) != 3 || quat.ndim() != 2 ||
                     quat.shape(0) < n || quat.shape(1) != 4)
                     throw py::value_error("need float32 arrays of shape (N, 3) and (N, 4)");
                 float* p = pos.mutable_data();
                 float* q = quat.mutable_data();
                 for (py::ssize_t i = 0; i < n; ++i) {
                     const Transform& t = s.transforms[(size_t)i];
                     p[3 * i] = t.position.x, p[3 * i + 1] = t.position.y, p[3 * i + 2] = t.position.z;
                     q[4 * i] = t.rotation.x, q[4 * i + 1] = t.rotation.y;
                     q[4 * i + 2] = t.rotation.z, q[4 * i + 3] = t.rotation.w;
                 }
             },
             py::arg("out_positions"), py::arg("out_quats"))
        .def_readonly("sleeping", &SimState::sleeping)
        .def_readonly("island_id", &SimState::island_id)
        .def("is_sleeping", &SimState::is_sleeping, py::arg("body_index"));

    py::class_<PhaseStat>(m, "PerformancePhaseStat")
        .def_readonly("name", &PhaseStat::name)
        .def_readonly("last_ms", &PhaseStat::last_ms)
        .def_readonly("avg_ms", &PhaseStat::avg_ms)
        .def_readonly("max_ms", &PhaseStat::max_ms)
        .def_readonly("samples", &PhaseStat::samples);
    py::class_<MetricValue>(m, "PerformanceMetric")
        .def_readonly("name", &MetricValue::name)
        .def_readonly("value", &MetricValue::value);
    py::class_<PerformanceMonitor>(m, "PerformanceMonitor")
        .def(py::init<>())
        .def_readwrite("enabled", &PerformanceMonitor::enabled)
        .def_readwrite("trace_enabled", &PerformanceMonitor::trace_enabled)
        .def_readwrite("trace_frame_capacity", &PerformanceMonitor::trace_frame_capacity)
        .def("write_trace_json",
             [](const PerformanceMonitor& m, const py::object& path) {
                 m.write_trace_json(py::str(path).cast<std::string>());
             },
             py::arg("path"))
        .def("phase_stats", &PerformanceMonitor::phase_stats)
        .def("last_frame_metrics", &PerformanceMonitor::last_frame_metrics)
        .def_property_readonly("frame_count", &PerformanceMonitor::frame_count)
        .def_property_readonly("last_frame_total_ms", &PerformanceMonitor::last_frame_total_ms)
        .def("reset", &PerformanceMonitor::reset);

    py::class_<World>(m, "World")
        .def(py::init<const Model&, SolverSettings>(), py::arg("model"),
             py::arg("solver_settings") = SolverSettings{})
        .def("step", &World::step, py::arg("dt"), py::call_guard<py::gil_scoped_release>())
        .def("set_gravity", &World::set_gravity, py::arg("gravity"))
        .def_property_readonly("gravity", &World::gravity)
        .def_property_readonly("state", &World::state, py::return_value_policy::reference_internal)
        .def_property_readonly("model", &World::model, py::return_value_policy::reference_internal)
        .def_property_readonly("contacts", &World::contacts)
        .def_property_readonly("performance_monitor", &World::performance_monitor,
                               py::return_value_policy::reference_internal)
        .def("apply_force", &World::apply_force, py::arg("body_index"), py::arg("force"))
        .def("apply_torque", &World::apply_torque, py::arg("body_index"), py::arg("torque"));

    // --- fluid (bind_fluid.cpp) ---
    py::class_<SPHKernels>(m, "SPHKernels")
        .def_static("poly6", &SPHKernels::poly6, py::arg("r_sq"), py::arg("h"))
        .def_static("spiky_grad", &SPHKernels::spiky_grad, py::arg("r"), py::arg("h"))
        .def_static("spiky", &SPHKernels::spiky, py::arg("r_len"), py::arg("h"))
        .def_static("cubic_spline", &SPHKernels::cubic_spline, py::arg("r_len"), py::arg("h"));

    py::class_<FluidBlockDef>(m, "FluidBlockDef")
        .def(py::init<>())
        .def_readwrite("lower", &FluidBlockDef::lower)
        .def_readwrite("upper", &FluidBlockDef::upper)
        .def_readwrite("particle_spacing", &FluidBlockDef::particle_spacing)
        .def_readwrite("rest_density", &FluidBlockDef::rest_density)
        .def_readwrite("initial_velocity", &FluidBlockDef::initial_velocity);

    py::class_<ParticleState>(m, "ParticleState")
        .def(py::init<>())
        .def("init", &ParticleState::init, py::arg("initial_positions"),
             py::arg("initial_velocity") = Vec3{})
        .def("clear", &ParticleState::clear)
        .def_property_readonly("num_particles", &ParticleState::num_particles)
        .def_readonly("positions", &ParticleState::positions)
        .def_readonly("velocities", &ParticleState::velocities)
        .def_readonly("densities", &ParticleState::densities)
        .def_readonly("lambdas", &ParticleState::lambdas)
        // (n, 3) / (n,) float32 array copies: one call instead of n Vector3 objects
        .def_property_readonly("positions_array",
                               [](const ParticleState& s) { return positions_array(s.positions); })
        .def_property_readonly("velocities_array",
                               [](const ParticleState& s) { return positions_array(s.velocities); })
        .def_property_readonly("densities_array", [](const ParticleState& s) {
            return py::array_t<float>((py::ssize_t)s.densities.size(), s.densities.data());
        })
        .def_property_readonly("lambdas_array", [](const ParticleState& s) {
            return py::array_t<float>((py::ssize_t)s.lambdas.size(), s.lambdas.data());
        });

    py::class_<SpatialHashGrid>(m, "SpatialHashGrid")
        .def(py::init<float>(), py::arg("cell_size") = 0.1f)
        .def("build", &SpatialHashGrid::build, py::arg("positions"))
        .def("clear", &SpatialHashGrid::clear)
        .def("query_neighbors", &SpatialHashGrid::query_neighbors, py::arg("point"),
             py::arg("radius"))
        .def("query_all_pairs", &SpatialHashGrid::query_all_pairs, py::arg("positions"),
             py::arg("radius"))
        .def_property("cell_size", &SpatialHashGrid::cell_size, &SpatialHashGrid::set_cell_size);

    py::class_<PBFSettings>(m, "PBFSettings")
        .def(py::init<>())
        .def_readwrite("rest_density", &PBFSettings::rest_density)
        .def_readwrite("kernel_radius", &PBFSettings::kernel_radius)
        .def_readwrite("particle_radius", &PBFSettings::particle_radius)
        .def_readwrite("solver_iterations", &PBFSettings::solver_iterations)
        .def_readwrite("epsilon", &PBFSettings::epsilon)
        .def_readwrite("xsph_viscosity", &PBFSettings::xsph_viscosity)
        .def_readwrite("vorticity_epsilon", &PBFSettings::vorticity_epsilon)
        .def_readwrite("corr_delta_q", &PBFSettings::corr_delta_q)
        .def_readwrite("corr_k", &PBFSettings::corr_k)
        .def_readwrite("corr_n", &PBFSettings::corr_n)
        .def_readwrite("use_domain_bounds", &PBFSettings::use_domain_bounds)
        .def_readwrite("domain_lower", &PBFSettings::domain_lower)
        .def_readwrite("domain_upper", &PBFSettings::domain_upper)
        .def_readwrite("exact_arithmetic", &PBFSettings::exact_arithmetic)
        .def_readwrite("hash_compat", &PBFSettings::hash_compat)
        .def_readwrite("boundary_two_way", &PBFSettings::boundary_two_way)
        .def_readwrite("boundary_friction", &PBFSettings::boundary_friction)
        .def("particle_mass", &PBFSettings::particle_mass, py::arg("spacing"));

    py::class_<PBFSolver>(m, "PBFSolver")
        .def(py::init<const PBFSettings&>(), py::arg("settings") = PBFSettings{})
        .def("step", &PBFSolver::step, py::arg("state"), py::arg("dt"), py::arg("gravity"),
             py::arg("particle_mass"), py::call_guard<py::gil_scoped_release>())
        .def_property_readonly("settings", &PBFSolver::settings,
                               py::return_value_policy::reference_internal);

    py::class_<BoundaryParticle>(m, "BoundaryParticle")
        .def(py::init<>())
        .def_readwrite("local_position", &BoundaryParticle::local_position)
        .def_readwrite("body_index", &BoundaryParticle::body_index)
        .def_readwrite("volume", &BoundaryParticle::volume);

    py::class_<FluidWorld, World>(m, "FluidWorld")
        .def(py::init<const Model&, const std::vector<FluidBlockDef>&, SolverSettings, PBFSettings,
                      float>(),
             py::arg("model"), py::arg("fluid_blocks") = std::vector<FluidBlockDef>{},
             py::arg("solver_settings") = SolverSettings{}, py::arg("pbf_settings") = PBFSettings{},
             py::arg("boundary_extent") = 1.0f)
        .def("step", &FluidWorld::step, py::arg("dt"), py::call_guard<py::gil_scoped_release>())
        .def_property_readonly("fluid_state", &FluidWorld::fluid_state,
                               py::return_value_policy::reference_internal)
        .def_property_readonly("num_particles", &FluidWorld::num_particles)
        .def_property_readonly("num_boundary_particles", &FluidWorld::num_boundary_particles)
        .def_property_readonly("boundary_particles", &FluidWorld::boundary_particles,
                               py::return_value_policy::reference_internal)
        .def_property_readonly("pbf_settings", &FluidWorld::pbf_settings,
                               py::return_value_policy::reference_internal)
        // Zero-copy state access (the reference's accessors copy into lists).
        .def(
            "fluid_arrays",
            [](py::object self) {
                FluidWorld& w = self.cast<FluidWorld&>();
                py::dict out;
                const py::ssize_t n = w.num_particles();
                for (int f = 0; f < 4; ++f) {
                    const float* p = w.fluid_pinned(f);
                    const bool vec = f < 2;
                    std::vector<py::ssize_t> shape = vec ? std::vector<py::ssize_t>{n, 3}
                                                         : std::vector<py::ssize_t>{n};
                    static float empty = 0.0f;
                    py::array_t<float> a(shape, p ? p : &empty, self);
                    a.attr("setflags")(py::arg("write") = false);
                    out[kFieldNames[f]] = a;
                }
                return out;
            },
            "The fluid state as numpy arrays that view page-locked host memory owned by the "
            "world: positions and velocities (n, 3), densities and lambdas (n,), float32. Each "
            "field is read from the device by one DMA, only when a step ran since its last "
            "read; the arrays are read-only views, so the next call after a step rewrites them "
            "in place.")
        .def(
            "fluid_device_arrays",
            [](py::object self) {
                FluidWorld& w = self.cast<FluidWorld&>();
                py::dict out;
                for (int f = 0; f < 4; ++f) {
                    DeviceFieldView v;
                    v.ptr = reinterpret_cast<uintptr_t>(w.fluid_device_field(f));
                    v.n = w.num_particles();
                    v.vec = f < 2;
                    v.owner = self;
                    out[kFieldNames[f]] = v;
                }
                return out;
            },
            "The fluid state in device memory as __cuda_array_interface__ views (no copy): "
            "positions and velocities (n, 3) with 16-byte rows, densities and lambdas (n,), "
            "float32, e.g. torch.as_tensor(view, device='cuda'). The world's stream is idle when "
            "this returns; later steps show through once they are synchronised.");

    py::class_<DeviceFieldView>(m, "DeviceFieldView")
        .def_property_readonly("__cuda_array_interface__", &DeviceFieldView::interface)
        .def_property_readonly("shape", [](const DeviceFieldView& v) -> py::tuple {
            if (v.vec) return py::make_tuple(v.n, 3);
            return py::make_tuple(v.n);
        });

    m.def("generate_fluid_block", &generate_fluid_block, py::arg("block_def"));
    m.def("sample_model_boundaries", &sample_model_boundaries, py::arg("model"),
          py::arg("spacing"), py::arg("plane_extent") = 1.0f);

    py::register_exception_translator([](std::exception_ptr p) {
        try {
            if (p) std::rethrow_exception(p);
        } catch (const std::invalid_argument& e) {
            PyErr_SetString(PyExc_ValueError, e.what());
        }
    });
}
