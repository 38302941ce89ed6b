// C-ABI harness around the reference's own PBF sources (test infrastructure
// only: the tests use it to pin the oracle restatement; the product never
// links it).  Built by oracle/build_oracle.py into oracle/_ref/ from the
// reference's unmodified files
//   src/fluid/pbf_solver.cpp, src/fluid/neighbor_search.cpp,
//   src/fluid/particle_state.cpp, src/sim/performance_monitor.cpp
// against the Eigen-API subset in oracle/eigen_shim (Eigen3 is absent here).
#include <cstring>
#include <vector>

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

}  // extern "C"
