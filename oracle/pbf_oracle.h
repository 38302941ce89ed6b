/*
 * CPU restatement of NovaPhy's PBF fluid step: the parity ORACLE.
 *
 * Test infrastructure only.  tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load it, and only as the checker; the product
 * (novaphy_gb300) never links or calls it.
 *
 * Parity is pinned: tests compare this restatement bit-for-bit against the
 * reference's own sources (src/fluid/pbf_solver.cpp, neighbor_search.cpp,
 * particle_state.cpp) compiled into oracle/_ref, and against the golden
 * fixtures under tests/golden generated from that build.  Vorticity
 * confinement has no reference implementation (the setting is never read);
 * its restatement follows Macklin & Mueller, "Position Based Fluids"
 * (SIGGRAPH 2013), section 5, and is unpinned.
 *
 * All arithmetic is float32 with no contraction (-ffp-contract=off), in the
 * reference's operation order.  A 3-term sum (squaredNorm, dot) is evaluated
 * as e0 + (e1 + e2).
 */
#ifndef NOVAPHY_PBF_ORACLE_H
#define NOVAPHY_PBF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Field order matches PBFSettings (include/novaphy/fluid/pbf_solver.h:13-38). */
typedef struct orc_settings {
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
} orc_settings;

void orc_default_settings(orc_settings* s);

/* Host threads of orc_pbf_step's per-particle loops (default 1); results do
 * not depend on it.  orc_max_threads: the processors OpenMP sees (1 when the
 * library was built without OpenMP). */
void orc_set_threads(int t);
int orc_max_threads(void);

/* SPH kernels, include/novaphy/fluid/sph_kernel.h:24-80. */
float orc_poly6(float r_sq, float h);
void orc_spiky_grad(const float* r, float h, float* out);
float orc_spiky(float r_len, float h);
float orc_cubic_spline(float r_len, float h);

/* Cell coordinates floor(p * (1/cell)), neighbor_search.cpp:99-105. */
void orc_cell_coords(const float* pts, int n, float cell, int* cells_out);

/* XOR-prime cell hash, neighbor_search.cpp:89-97. */
unsigned long long orc_hash_cell(int cx, int cy, int cz);

/* Candidate list of a query point over a hash grid built on `pts` (order of
 * SpatialHashGrid::query_neighbors, neighbor_search.cpp:28-49).  Writes up to
 * `cap` indices and returns the full count (-1 on allocation failure). */
int orc_grid_query(const float* pts, int n, float cell, const float* q, int* out, int cap);

/* Number of particles whose 27-cell neighbourhood holds two distinct cells
 * with equal hash keys (0 means the hashed grid gives the same candidate
 * sums as a dense grid). */
int orc_hash_collisions(const float* pts, int n, float cell);

/* Canonical neighbour sets at the predicted positions of the step start:
 * for particle i, the sorted {j != i : candidate of i and |x*_i - x*_j|^2 < h*h}.
 * offsets has n+1 entries; returns the total count or -1 on failure.  Pass
 * out=NULL to size (the sizing count includes repeats from double-visited
 * buckets; the filled sets are deduplicated and the offsets/total describe
 * them). */
long long orc_neighbor_sets(const float* xs, int n, float h, long long* offsets, int* out,
                            long long cap);

/* One full PBF step (pbf_solver.cpp:18-127) plus, when
 * vorticity_epsilon > 0, the project's vorticity confinement.  x, v: n*3 in
 * place; rho, lam: n in place.  Returns 0, or -1 on allocation failure. */
int orc_pbf_step(const orc_settings* s, int n, float* x, float* v, float* rho, float* lam,
                 float dt, const float* g, float mass);

/* Predicted positions after `predict` only (pbf_solver.cpp:28-34). */
void orc_predict(int n, const float* x, const float* v, float dt, const float* g, float* xs_out,
                 float* v_out);

/* ---- Akinci boundary handling (src/fluid/boundary.cpp, fluid_world.cpp) ---- */

/* x_b = T[body] * local (quaternion w,x,y,z), boundary.cpp:178-192. */
void orc_boundary_world_positions(int nb, const float* local3, const int* body, int nbodies,
                                  const float* body_pos3, const float* body_quat4, float* out3);

/* psi_b = 1 / sum_b' poly6, boundary.cpp:152-176.  Returns -1 on failure. */
int orc_boundary_volumes(int nb, const float* world3, float h, float* psi_out);

/* rho_i += sum_b rho0 psi_b poly6(|x_i - x_b|^2), fluid_world.cpp:101-123. */
int orc_boundary_density(int n, const float* x3, float* rho, int nb, const float* bpos3,
                         const float* psi, float h, float rho0);

/* Per-body force and torque from fluid pressure, fluid_world.cpp:125-174.
 * body_dynamic[k] != 0 marks dynamic bodies.  force3/torque3 have nbodies*3
 * entries and are ACCUMULATED into (like World::apply_force). */
int orc_coupling_forces(int n, const float* x3, const float* rho, float mass, int nb,
                        const float* bpos3, const int* body, const float* psi, int nbodies,
                        const int* body_dynamic, const float* body_pos3, float h, float rho0,
                        float* force3, float* torque3);

/* Boundary sampling, boundary.cpp:15-126.  The local transform is given as
 * position + quaternion (w,x,y,z).  Each returns the count and writes up to
 * `cap` local positions. */
int orc_sample_box(const float* half_extents, const float* lt_pos, const float* lt_quat,
                   float spacing, float* out3, int cap);
int orc_sample_sphere(float radius, const float* lt_pos, const float* lt_quat, float spacing,
                      float* out3, int cap);
int orc_sample_plane(const float* normal, float offset, float spacing, float extent, float* out3,
                     int cap);

/* generate_fluid_block, particle_state.cpp:31-58. */
int orc_generate_block(const float* lower, const float* upper, float spacing, float* out3,
                       int cap);

#ifdef __cplusplus
}
#endif

#endif
