/*
 * CPU restatement of NovaPhy's PBF fluid step: the parity ORACLE.
 * Test infrastructure only (see pbf_oracle.h for who may call it).
 *
 * Every function cites the reference lines it restates.  Build with
 * -O2 -ffp-contract=off so that no multiply-add is fused: the operation order
 * below is the reference's, term by term.
 */
#include "pbf_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Host threads of the per-particle loops of orc_pbf_step (1 by default, as
 * the reference is single-threaded).  Every particle's sums keep their
 * sequential order, so results do not depend on the thread count. */
static int g_threads = 1;

void orc_set_threads(int t) { g_threads = t > 0 ? t : 1; }

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_num_procs();
#else
    return 1;
#endif
}

#ifdef _OPENMP
#define ORC_PARALLEL_FOR _Pragma("omp parallel for schedule(dynamic, 512) num_threads(g_threads)")
#else
#define ORC_PARALLEL_FOR
#endif

#define ORC_PI 3.14159265358979323846f /* math_utils.h:53 */

/* e0 + (e1 + e2): 3-term reduction order (squaredNorm / dot). */
static inline float sum3(float a, float b, float c) { return a + (b + c); }
static inline float sqn3(float x, float y, float z) { return sum3(x * x, y * y, z * z); }

void orc_default_settings(orc_settings* s) {
    /* pbf_solver.h:14-27 */
    s->rest_density = 1000.0f;
    s->kernel_radius = 0.1f;
    s->particle_radius = 0.025f;
    s->solver_iterations = 4;
    s->epsilon = 100.0f;
    s->xsph_viscosity = 0.01f;
    s->vorticity_epsilon = 0.0f;
    s->corr_delta_q = 0.3f;
    s->corr_k = 0.001f;
    s->corr_n = 4;
    s->use_domain_bounds = 0;
    s->domain_lower[0] = -10.0f;
    s->domain_lower[1] = 0.0f;
    s->domain_lower[2] = -10.0f;
    s->domain_upper[0] = 10.0f;
    s->domain_upper[1] = 10.0f;
    s->domain_upper[2] = 10.0f;
}

/* ---------------- SPH kernels: sph_kernel.h:24-80 ---------------- */

float orc_poly6(float r_sq, float h) {
    /* sph_kernel.h:24-30 */
    if (r_sq >= h * h) return 0.0f;
    float h2 = h * h;
    float diff = h2 - r_sq;
    float h9 = h2 * h2 * h2 * h2 * h;
    return (315.0f / (64.0f * ORC_PI * h9)) * diff * diff * diff;
}

static inline void spiky_grad3(float rx, float ry, float rz, float h, float* gx, float* gy,
                               float* gz) {
    /* sph_kernel.h:39-46 */
    float r_len = sqrtf(sqn3(rx, ry, rz));
    if (r_len <= 1e-7f || r_len >= h) {
        *gx = 0.0f;
        *gy = 0.0f;
        *gz = 0.0f;
        return;
    }
    float diff = h - r_len;
    float h6 = h * h * h * h * h * h;
    float coeff = -(45.0f / (ORC_PI * h6)) * diff * diff / r_len;
    *gx = coeff * rx;
    *gy = coeff * ry;
    *gz = coeff * rz;
}

void orc_spiky_grad(const float* r, float h, float* out) {
    spiky_grad3(r[0], r[1], r[2], h, &out[0], &out[1], &out[2]);
}

float orc_spiky(float r_len, float h) {
    /* sph_kernel.h:55-60 */
    if (r_len >= h || r_len < 0.0f) return 0.0f;
    float diff = h - r_len;
    float h6 = h * h * h * h * h * h;
    return (15.0f / (ORC_PI * h6)) * diff * diff * diff;
}

float orc_cubic_spline(float r_len, float h) {
    /* sph_kernel.h:69-80 */
    float q = r_len / h;
    if (q >= 1.0f) return 0.0f;
    float h3 = h * h * h;
    float sigma = 8.0f / (ORC_PI * h3);
    if (q <= 0.5f) return sigma * (6.0f * (q * q * q - q * q) + 1.0f);
    float t = 1.0f - q;
    return sigma * 2.0f * t * t * t;
}

/* ---------------- spatial hash grid: neighbor_search.cpp ---------------- */

unsigned long long orc_hash_cell(int cx, int cy, int cz) {
    /* neighbor_search.cpp:89-97: sign-extended int -> uint64, XOR of products */
    const uint64_t p1 = 73856093ULL, p2 = 19349663ULL, p3 = 83492791ULL;
    return ((uint64_t)(int64_t)cx * p1) ^ ((uint64_t)(int64_t)cy * p2) ^
           ((uint64_t)(int64_t)cz * p3);
}

static inline void world_to_cell(const float* p, float inv, int* c) {
    /* neighbor_search.cpp:99-105 */
    c[0] = (int)floorf(p[0] * inv);
    c[1] = (int)floorf(p[1] * inv);
    c[2] = (int)floorf(p[2] * inv);
}

void orc_cell_coords(const float* pts, int n, float cell, int* cells_out) {
    float inv = 1.0f / cell;
    for (int i = 0; i < n; ++i) world_to_cell(pts + 3 * i, inv, cells_out + 3 * i);
}

/* A built grid: (key, index) pairs sorted by key then index.  A bucket is a
 * run of equal keys, holding indices in ascending order exactly like the
 * reference's unordered_map<key, vector<int>> filled in index order
 * (neighbor_search.cpp:14-22). */
typedef struct {
    uint64_t key;
    int idx;
} kv_t;

typedef struct {
    kv_t* kv;
    int n;
    float inv;
} grid_t;

static int kv_cmp(const void* a, const void* b) {
    const kv_t* x = (const kv_t*)a;
    const kv_t* y = (const kv_t*)b;
    if (x->key < y->key) return -1;
    if (x->key > y->key) return 1;
    return (x->idx > y->idx) - (x->idx < y->idx);
}

static int grid_build(grid_t* g, const float* pts, int n, float cell) {
    g->n = n;
    g->inv = 1.0f / cell;
    g->kv = (kv_t*)malloc(sizeof(kv_t) * (size_t)(n > 0 ? n : 1));
    if (!g->kv) return -1;
    for (int i = 0; i < n; ++i) {
        int c[3];
        world_to_cell(pts + 3 * i, g->inv, c);
        g->kv[i].key = orc_hash_cell(c[0], c[1], c[2]);
        g->kv[i].idx = i;
    }
    qsort(g->kv, (size_t)n, sizeof(kv_t), kv_cmp);
    return 0;
}

static void grid_free(grid_t* g) { free(g->kv); }

/* Bucket [*lo, *hi) of `key` in the sorted pairs. */
static void grid_bucket(const grid_t* g, uint64_t key, int* lo, int* hi) {
    int a = 0, b = g->n;
    while (a < b) {
        int m = a + (b - a) / 2;
        if (g->kv[m].key < key) a = m + 1;
        else b = m;
    }
    int s = a;
    b = g->n;
    while (a < b) {
        int m = a + (b - a) / 2;
        if (g->kv[m].key <= key) a = m + 1;
        else b = m;
    }
    *lo = s;
    *hi = a;
}

/* Candidate list of cell c: 27 buckets in dz, dy, dx order
 * (neighbor_search.cpp:36-48).  Returns the count; writes up to cap. */
static int grid_candidates(const grid_t* g, const int* c, int* out, int cap) {
    int m = 0;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                int lo, hi;
                grid_bucket(g, orc_hash_cell(c[0] + dx, c[1] + dy, c[2] + dz), &lo, &hi);
                for (int k = lo; k < hi; ++k) {
                    if (m < cap) out[m] = g->kv[k].idx;
                    ++m;
                }
            }
    return m;
}

/* Candidate list of cell c into *buf (grown as needed: with double-visited
 * buckets a list can be longer than the point count). Returns the count or
 * -1 on allocation failure. */
static int grid_candidates_buf(const grid_t* g, const int* c, int** buf, int* cap) {
    int m = grid_candidates(g, c, NULL, 0);
    if (m > *cap) {
        int* nb = (int*)realloc(*buf, sizeof(int) * (size_t)m);
        if (!nb) return -1;
        *buf = nb;
        *cap = m;
    }
    grid_candidates(g, c, *buf, *cap);
    return m;
}

int orc_grid_query(const float* pts, int n, float cell, const float* q, int* out, int cap) {
    grid_t g;
    if (grid_build(&g, pts, n, cell)) return -1;
    int c[3];
    world_to_cell(q, g.inv, c);
    int m = grid_candidates(&g, c, out, cap);
    grid_free(&g);
    return m;
}

static int u64_cmp(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return (x > y) - (x < y);
}

int orc_hash_collisions(const float* pts, int n, float cell) {
    /* Number of particles whose 27 neighbour cells (neighbor_search.cpp:36-48)
     * contain two distinct cells with the same hash key.  Such a particle
     * would see one bucket twice in the reference (double counting); any
     * other key collision only merges a far cell whose particles are beyond
     * the kernel radius and add exact zeros. */
    float inv = 1.0f / cell;
    int bad = 0;
    for (int i = 0; i < n; ++i) {
        int c[3];
        uint64_t keys[27];
        world_to_cell(pts + 3 * i, inv, c);
        int k = 0;
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx)
                    keys[k++] = orc_hash_cell(c[0] + dx, c[1] + dy, c[2] + dz);
        qsort(keys, 27, sizeof(uint64_t), u64_cmp);
        for (k = 1; k < 27; ++k)
            if (keys[k] == keys[k - 1]) {
                ++bad;
                break;
            }
    }
    return bad;
}

/* ---------------- PBF step: pbf_solver.cpp ---------------- */

void orc_predict(int n, const float* x, const float* v, float dt, const float* g, float* xs_out,
                 float* v_out) {
    /* pbf_solver.cpp:30-33 */
    for (int i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c) {
            float vc = v[3 * i + c] + g[c] * dt;
            v_out[3 * i + c] = vc;
            xs_out[3 * i + c] = x[3 * i + c] + vc * dt;
        }
}

long long orc_neighbor_sets(const float* xs, int n, float h, long long* offsets, int* out,
                            long long cap) {
    grid_t g;
    if (grid_build(&g, xs, n, h)) return -1;
    int ccap = n > 0 ? n : 1;
    int* cand = (int*)malloc(sizeof(int) * (size_t)ccap);
    if (!cand) {
        grid_free(&g);
        return -1;
    }
    long long tot = 0;
    float hh = h * h;
    for (int i = 0; i < n; ++i) {
        int c[3];
        world_to_cell(xs + 3 * i, g.inv, c);
        int m = grid_candidates_buf(&g, c, &cand, &ccap);
        if (m < 0) {
            free(cand);
            grid_free(&g);
            return -1;
        }
        if (offsets) offsets[i] = tot;
        /* Candidate lists are sorted by (bucket, index); gather the in-radius
         * ones and sort ascending for the canonical set. */
        long long start = tot;
        for (int k = 0; k < m; ++k) {
            int j = cand[k];
            if (j == i) continue;
            float rx = xs[3 * i] - xs[3 * j];
            float ry = xs[3 * i + 1] - xs[3 * j + 1];
            float rz = xs[3 * i + 2] - xs[3 * j + 2];
            if (sqn3(rx, ry, rz) < hh) {
                if (out && tot < cap) out[tot] = j;
                ++tot;
            }
        }
        if (out && tot <= cap) {
            /* insertion sort of the (short) set, then drop the repeats that
             * double-visited buckets produce: a canonical set */
            for (long long a = start + 1; a < tot; ++a) {
                int v = out[a];
                long long b = a - 1;
                while (b >= start && out[b] > v) {
                    out[b + 1] = out[b];
                    --b;
                }
                out[b + 1] = v;
            }
            long long w = start;
            for (long long a = start; a < tot; ++a)
                if (a == start || out[a] != out[w - 1]) out[w++] = out[a];
            tot = w;
        }
    }
    if (offsets) offsets[n] = tot;
    free(cand);
    grid_free(&g);
    return tot;
}

/* Candidate table of one step: per particle, the candidate list computed once
 * at step start from the grid on x* (pbf_solver.cpp:43-51). */
typedef struct {
    int* idx;
    long long* off;
} cand_t;

static int build_candidates(cand_t* ct, const float* xs, int n, float h) {
    grid_t g;
    if (grid_build(&g, xs, n, h)) return -1;
    ct->off = (long long*)malloc(sizeof(long long) * (size_t)(n + 1));
    if (!ct->off) {
        grid_free(&g);
        return -1;
    }
    ORC_PARALLEL_FOR
    for (int i = 0; i < n; ++i) {
        int c[3];
        world_to_cell(xs + 3 * i, g.inv, c);
        ct->off[i + 1] = grid_candidates(&g, c, NULL, 0);
    }
    long long tot = 0;
    for (int i = 0; i < n; ++i) {
        long long m = ct->off[i + 1];
        ct->off[i] = tot;
        tot += m;
    }
    ct->off[n] = tot;
    ct->idx = (int*)malloc(sizeof(int) * (size_t)(tot > 0 ? tot : 1));
    if (!ct->idx) {
        free(ct->off);
        grid_free(&g);
        return -1;
    }
    ORC_PARALLEL_FOR
    for (int i = 0; i < n; ++i) {
        int c[3];
        world_to_cell(xs + 3 * i, g.inv, c);
        grid_candidates(&g, c, ct->idx + ct->off[i], (int)(ct->off[i + 1] - ct->off[i]));
    }
    grid_free(&g);
    return 0;
}

static void free_candidates(cand_t* ct) {
    free(ct->idx);
    free(ct->off);
}

static void compute_density(const cand_t* ct, int n, const float* xs, float* rho, float mass,
                            float h) {
    /* pbf_solver.cpp:129-142 (self included) */
    ORC_PARALLEL_FOR
    for (int i = 0; i < n; ++i) {
        float density = 0.0f;
        for (long long k = ct->off[i]; k < ct->off[i + 1]; ++k) {
            int j = ct->idx[k];
            float rx = xs[3 * i] - xs[3 * j];
            float ry = xs[3 * i + 1] - xs[3 * j + 1];
            float rz = xs[3 * i + 2] - xs[3 * j + 2];
            float r_sq = sqn3(rx, ry, rz);
            density += mass * orc_poly6(r_sq, h);
        }
        rho[i] = density;
    }
}

static void compute_lambda(const cand_t* ct, int n, const float* xs, const float* rho,
                           float* lam, float mass, const orc_settings* s) {
    /* pbf_solver.cpp:144-179 */
    float h = s->kernel_radius;
    float rho0 = s->rest_density;
    float eps = s->epsilon;
    float inv_rho0 = 1.0f / rho0;
    ORC_PARALLEL_FOR
    for (int i = 0; i < n; ++i) {
        float C_i = rho[i] * inv_rho0 - 1.0f;
        if (C_i < 0.0f) {
            lam[i] = 0.0f;
            continue;
        }
        float sum_grad_sq = 0.0f;
        float gi[3] = {0.0f, 0.0f, 0.0f};
        float mr = mass * inv_rho0;
        for (long long k = ct->off[i]; k < ct->off[i + 1]; ++k) {
            int j = ct->idx[k];
            if (j == i) continue;
            float g[3];
            spiky_grad3(xs[3 * i] - xs[3 * j], xs[3 * i + 1] - xs[3 * j + 1],
                        xs[3 * i + 2] - xs[3 * j + 2], h, &g[0], &g[1], &g[2]);
            float gj0 = mr * g[0], gj1 = mr * g[1], gj2 = mr * g[2];
            sum_grad_sq += sqn3(gj0, gj1, gj2);
            gi[0] += gj0;
            gi[1] += gj1;
            gi[2] += gj2;
        }
        sum_grad_sq += sqn3(gi[0], gi[1], gi[2]);
        lam[i] = -C_i / (sum_grad_sq + eps);
    }
}

static void compute_delta_position(const cand_t* ct, int n, const float* xs, const float* lam,
                                   float* dp, float mass, const orc_settings* s) {
    /* pbf_solver.cpp:181-223 */
    float h = s->kernel_radius;
    float rho0 = s->rest_density;
    float inv_rho0 = 1.0f / rho0;
    float delta_q = s->corr_delta_q * h;
    float w_delta_q = orc_poly6(delta_q * delta_q, h);
    ORC_PARALLEL_FOR
    for (int i = 0; i < n; ++i) {
        float d[3] = {0.0f, 0.0f, 0.0f};
        for (long long k = ct->off[i]; k < ct->off[i + 1]; ++k) {
            int j = ct->idx[k];
            if (j == i) continue;
            float rx = xs[3 * i] - xs[3 * j];
            float ry = xs[3 * i + 1] - xs[3 * j + 1];
            float rz = xs[3 * i + 2] - xs[3 * j + 2];
            float r_sq = sqn3(rx, ry, rz);
            float lambda_sum = lam[i] + lam[j];
            float s_corr = 0.0f;
            if (lambda_sum < -1e-10f && w_delta_q > 1e-10f) {
                float ratio = orc_poly6(r_sq, h) / w_delta_q;
                ratio = (1.0f < ratio) ? 1.0f : ratio; /* std::min(ratio, 1.0f) */
                float ratio_pow = ratio * ratio;
                if (s->corr_n == 4) ratio_pow = ratio_pow * ratio_pow;
                s_corr = -s->corr_k * ratio_pow;
            }
            float g[3];
            spiky_grad3(rx, ry, rz, h, &g[0], &g[1], &g[2]);
            float a = (lambda_sum + s_corr) * mass;
            d[0] += a * g[0];
            d[1] += a * g[1];
            d[2] += a * g[2];
        }
        dp[3 * i] = d[0] * inv_rho0;
        dp[3 * i + 1] = d[1] * inv_rho0;
        dp[3 * i + 2] = d[2] * inv_rho0;
    }
}

/* Vorticity confinement (no reference implementation: PBFSettings::
 * vorticity_epsilon, pbf_solver.h:20, is never read).  Restated from
 * Macklin & Mueller 2013, section 5, with the velocities after the velocity
 * update (the same input XSPH reads):
 *   omega_i = sum_{j!=i} (m / rho_j') spiky_grad(x*_i - x*_j) x (v_j - v_i)
 *   eta_i   = sum_{j!=i} (m / rho_j') (|omega_j| - |omega_i|) spiky_grad(x*_i - x*_j)
 *   N_i     = eta_i / |eta_i|   (0 when |eta_i| <= 1e-9)
 *   v_i    += dt * eps_v * (N_i x omega_i)
 * with rho_j' = rho_j if rho_j > 1e-6 else rho0 (the XSPH density guard).
 * The curl estimate carries the SPH volume m / rho_j' (the paper's formula
 * omits it), so omega is in 1/s and eps_v in m/s.  The increment is added
 * after the XSPH correction. */
static void vorticity_omega(const cand_t* ct, int n, const float* xs, const float* v,
                            const float* rho, float mass, float rho0, float h, float* omega) {
    ORC_PARALLEL_FOR
    for (int i = 0; i < n; ++i) {
        float w[3] = {0.0f, 0.0f, 0.0f};
        for (long long k = ct->off[i]; k < ct->off[i + 1]; ++k) {
            int j = ct->idx[k];
            if (j == i) continue;
            float g[3];
            spiky_grad3(xs[3 * i] - xs[3 * j], xs[3 * i + 1] - xs[3 * j + 1],
                        xs[3 * i + 2] - xs[3 * j + 2], h, &g[0], &g[1], &g[2]);
            float u0 = v[3 * j] - v[3 * i];
            float u1 = v[3 * j + 1] - v[3 * i + 1];
            float u2 = v[3 * j + 2] - v[3 * i + 2];
            float rho_j = (rho[j] > 1e-6f) ? rho[j] : rho0;
            float f = mass / rho_j;
            w[0] += f * (g[1] * u2 - g[2] * u1);
            w[1] += f * (g[2] * u0 - g[0] * u2);
            w[2] += f * (g[0] * u1 - g[1] * u0);
        }
        omega[3 * i] = w[0];
        omega[3 * i + 1] = w[1];
        omega[3 * i + 2] = w[2];
    }
}

static void vorticity_apply(const cand_t* ct, int n, const float* xs, const float* rho,
                            const float* omega, float mass, const orc_settings* s, float dt,
                            float* dv) {
    float h = s->kernel_radius;
    float rho0 = s->rest_density;
    float eps_v = s->vorticity_epsilon;
    ORC_PARALLEL_FOR
    for (int i = 0; i < n; ++i) {
        float wi = sqrtf(sqn3(omega[3 * i], omega[3 * i + 1], omega[3 * i + 2]));
        float eta[3] = {0.0f, 0.0f, 0.0f};
        for (long long k = ct->off[i]; k < ct->off[i + 1]; ++k) {
            int j = ct->idx[k];
            if (j == i) continue;
            float g[3];
            spiky_grad3(xs[3 * i] - xs[3 * j], xs[3 * i + 1] - xs[3 * j + 1],
                        xs[3 * i + 2] - xs[3 * j + 2], h, &g[0], &g[1], &g[2]);
            float wj = sqrtf(sqn3(omega[3 * j], omega[3 * j + 1], omega[3 * j + 2]));
            float rho_j = (rho[j] > 1e-6f) ? rho[j] : rho0;
            float a = (mass / rho_j) * (wj - wi);
            eta[0] += a * g[0];
            eta[1] += a * g[1];
            eta[2] += a * g[2];
        }
        float el = sqrtf(sqn3(eta[0], eta[1], eta[2]));
        float N[3] = {0.0f, 0.0f, 0.0f};
        if (el > 1e-9f) {
            N[0] = eta[0] / el;
            N[1] = eta[1] / el;
            N[2] = eta[2] / el;
        }
        float f0 = N[1] * omega[3 * i + 2] - N[2] * omega[3 * i + 1];
        float f1 = N[2] * omega[3 * i] - N[0] * omega[3 * i + 2];
        float f2 = N[0] * omega[3 * i + 1] - N[1] * omega[3 * i];
        float sc = dt * eps_v;
        dv[3 * i] = sc * f0;
        dv[3 * i + 1] = sc * f1;
        dv[3 * i + 2] = sc * f2;
    }
}

int orc_pbf_step(const orc_settings* s, int n, float* x, float* v, float* rho, float* lam,
                 float dt, const float* g, float mass) {
    /* pbf_solver.cpp:18-127 */
    if (n == 0) return 0;
    float h = s->kernel_radius;
    size_t n3 = (size_t)n * 3;
    float* xs = (float*)malloc(sizeof(float) * n3);
    float* dp = (float*)malloc(sizeof(float) * n3);
    float* vv = (float*)malloc(sizeof(float) * n3);
    float* om = (float*)malloc(sizeof(float) * n3);
    float* dv = (float*)malloc(sizeof(float) * n3);
    if (!xs || !dp || !vv || !om || !dv) {
        free(xs), free(dp), free(vv), free(om), free(dv);
        return -1;
    }
    /* 1. predict */
    orc_predict(n, x, v, dt, g, xs, v);
    /* 2-3. grid + fixed candidate lists */
    cand_t ct;
    if (build_candidates(&ct, xs, n, h)) {
        free(xs), free(dp), free(vv), free(om), free(dv);
        return -1;
    }
    /* 4. Jacobi iterations */
    for (int it = 0; it < s->solver_iterations; ++it) {
        compute_density(&ct, n, xs, rho, mass, h);
        compute_lambda(&ct, n, xs, rho, lam, mass, s);
        compute_delta_position(&ct, n, xs, lam, dp, mass, s);
        for (size_t k = 0; k < n3; ++k) xs[k] += dp[k];
    }
    /* 5. velocity update with clamp, pbf_solver.cpp:81-93 */
    float inv_dt = 1.0f / dt;
    float max_speed = h / dt;
    float max_speed_sq = max_speed * max_speed;
    ORC_PARALLEL_FOR
    for (int i = 0; i < n; ++i) {
        float a = (xs[3 * i] - x[3 * i]) * inv_dt;
        float b = (xs[3 * i + 1] - x[3 * i + 1]) * inv_dt;
        float c = (xs[3 * i + 2] - x[3 * i + 2]) * inv_dt;
        float speed_sq = sqn3(a, b, c);
        if (speed_sq > max_speed_sq) {
            float sc = max_speed / sqrtf(speed_sq);
            a *= sc;
            b *= sc;
            c *= sc;
        }
        v[3 * i] = a;
        v[3 * i + 1] = b;
        v[3 * i + 2] = c;
    }
    /* vorticity input is the post-update velocity */
    int vort = s->vorticity_epsilon > 0.0f;
    if (vort) vorticity_omega(&ct, n, xs, v, rho, mass, s->rest_density, h, om);
    /* 6. XSPH, pbf_solver.cpp:225-250 */
    if (s->xsph_viscosity > 0.0f) {
        float cx = s->xsph_viscosity;
        float rho0 = s->rest_density;
        ORC_PARALLEL_FOR
        for (int i = 0; i < n; ++i) {
            float vc[3] = {0.0f, 0.0f, 0.0f};
            for (long long k = ct.off[i]; k < ct.off[i + 1]; ++k) {
                int j = ct.idx[k];
                if (j == i) continue;
                float u0 = v[3 * j] - v[3 * i];
                float u1 = v[3 * j + 1] - v[3 * i + 1];
                float u2 = v[3 * j + 2] - v[3 * i + 2];
                float rx = xs[3 * i] - xs[3 * j];
                float ry = xs[3 * i + 1] - xs[3 * j + 1];
                float rz = xs[3 * i + 2] - xs[3 * j + 2];
                float w = orc_poly6(sqn3(rx, ry, rz), h);
                float rho_j = (rho[j] > 1e-6f) ? rho[j] : rho0;
                float f = mass / rho_j;
                vc[0] += f * u0 * w;
                vc[1] += f * u1 * w;
                vc[2] += f * u2 * w;
            }
            vv[3 * i] = vc[0];
            vv[3 * i + 1] = vc[1];
            vv[3 * i + 2] = vc[2];
        }
    }
    if (vort) vorticity_apply(&ct, n, xs, rho, om, mass, s, dt, dv);
    if (s->xsph_viscosity > 0.0f)
        for (size_t k = 0; k < n3; ++k) v[k] += s->xsph_viscosity * vv[k];
    if (vort)
        for (size_t k = 0; k < n3; ++k) v[k] += dv[k];
    /* 7. commit with optional domain clamp, pbf_solver.cpp:102-126 */
    if (s->use_domain_bounds) {
        float pr = s->particle_radius;
        float lo[3], hi[3];
        for (int d = 0; d < 3; ++d) {
            lo[d] = s->domain_lower[d] + pr;
            hi[d] = s->domain_upper[d] - pr;
        }
        for (int i = 0; i < n; ++i)
            for (int d = 0; d < 3; ++d) {
                float p = xs[3 * i + d];
                if (p < lo[d]) {
                    p = lo[d];
                    v[3 * i + d] = 0.0f;
                } else if (p > hi[d]) {
                    p = hi[d];
                    v[3 * i + d] = 0.0f;
                }
                x[3 * i + d] = p;
            }
    } else {
        memcpy(x, xs, sizeof(float) * n3);
    }
    free_candidates(&ct);
    free(xs), free(dp), free(vv), free(om), free(dv);
    return 0;
}

/* ---------------- Akinci boundary: boundary.cpp / fluid_world.cpp ---------------- */

/* Quaternion (w,x,y,z) rotation of p: t = 2 (q.vec x p); p + w t + q.vec x t. */
static void quat_rotate(const float* q, const float* p, float* out) {
    float w = q[0], qx = q[1], qy = q[2], qz = q[3];
    float t0 = qy * p[2] - qz * p[1];
    float t1 = qz * p[0] - qx * p[2];
    float t2 = qx * p[1] - qy * p[0];
    t0 = t0 + t0;
    t1 = t1 + t1;
    t2 = t2 + t2;
    float c0 = qy * t2 - qz * t1;
    float c1 = qz * t0 - qx * t2;
    float c2 = qx * t1 - qy * t0;
    out[0] = (p[0] + w * t0) + c0;
    out[1] = (p[1] + w * t1) + c1;
    out[2] = (p[2] + w * t2) + c2;
}

static void transform_point(const float* pos, const float* q, const float* p, float* out) {
    /* math_types.h:80: position + rotation * p */
    float r[3];
    quat_rotate(q, p, r);
    out[0] = pos[0] + r[0];
    out[1] = pos[1] + r[1];
    out[2] = pos[2] + r[2];
}

void orc_boundary_world_positions(int nb, const float* local3, const int* body, int nbodies,
                                  const float* body_pos3, const float* body_quat4, float* out3) {
    /* boundary.cpp:178-192 */
    for (int i = 0; i < nb; ++i) {
        int bi = body[i];
        if (bi >= 0 && bi < nbodies)
            transform_point(body_pos3 + 3 * bi, body_quat4 + 4 * bi, local3 + 3 * i, out3 + 3 * i);
        else
            memcpy(out3 + 3 * i, local3 + 3 * i, sizeof(float) * 3);
    }
}

int orc_boundary_volumes(int nb, const float* world3, float h, float* psi_out) {
    /* boundary.cpp:152-176 */
    if (nb == 0) return 0;
    grid_t g;
    if (grid_build(&g, world3, nb, h)) return -1;
    int ccap = nb;
    int* cand = (int*)malloc(sizeof(int) * (size_t)ccap);
    if (!cand) {
        grid_free(&g);
        return -1;
    }
    for (int i = 0; i < nb; ++i) {
        int c[3];
        world_to_cell(world3 + 3 * i, g.inv, c);
        int m = grid_candidates_buf(&g, c, &cand, &ccap);
        if (m < 0) {
            free(cand);
            grid_free(&g);
            return -1;
        }
        float sum_w = 0.0f;
        for (int k = 0; k < m; ++k) {
            int j = cand[k];
            float rx = world3[3 * i] - world3[3 * j];
            float ry = world3[3 * i + 1] - world3[3 * j + 1];
            float rz = world3[3 * i + 2] - world3[3 * j + 2];
            sum_w += orc_poly6(sqn3(rx, ry, rz), h);
        }
        psi_out[i] = (sum_w > 1e-10f) ? 1.0f / sum_w : 0.0f;
    }
    free(cand);
    grid_free(&g);
    return 0;
}

int orc_boundary_density(int n, const float* x3, float* rho, int nb, const float* bpos3,
                         const float* psi, float h, float rho0) {
    /* fluid_world.cpp:101-123 */
    if (nb == 0 || n == 0) return 0;
    grid_t g;
    if (grid_build(&g, bpos3, nb, h)) return -1;
    int ccap = nb;
    int* cand = (int*)malloc(sizeof(int) * (size_t)ccap);
    if (!cand) {
        grid_free(&g);
        return -1;
    }
    for (int i = 0; i < n; ++i) {
        int c[3];
        world_to_cell(x3 + 3 * i, g.inv, c);
        int m = grid_candidates_buf(&g, c, &cand, &ccap);
        if (m < 0) {
            free(cand);
            grid_free(&g);
            return -1;
        }
        float bd = 0.0f;
        for (int k = 0; k < m; ++k) {
            int j = cand[k];
            float rx = x3[3 * i] - bpos3[3 * j];
            float ry = x3[3 * i + 1] - bpos3[3 * j + 1];
            float rz = x3[3 * i + 2] - bpos3[3 * j + 2];
            bd += rho0 * psi[j] * orc_poly6(sqn3(rx, ry, rz), h);
        }
        rho[i] += bd;
    }
    free(cand);
    grid_free(&g);
    return 0;
}

int orc_coupling_forces(int n, const float* x3, const float* rho, float mass, int nb,
                        const float* bpos3, const int* body, const float* psi, int nbodies,
                        const int* body_dynamic, const float* body_pos3, float h, float rho0,
                        float* force3, float* torque3) {
    /* fluid_world.cpp:125-174 */
    if (nb == 0 || n == 0) return 0;
    grid_t g;
    if (grid_build(&g, x3, n, h)) return -1;
    int ccap = n;
    int* cand = (int*)malloc(sizeof(int) * (size_t)ccap);
    if (!cand) {
        grid_free(&g);
        return -1;
    }
    float hh = h * h;
    for (int b = 0; b < nb; ++b) {
        int bi = body[b];
        if (bi < 0) continue;
        if (bi >= nbodies || !body_dynamic[bi]) continue;
        float f[3] = {0.0f, 0.0f, 0.0f};
        float psi_b = psi[b];
        int c[3];
        world_to_cell(bpos3 + 3 * b, g.inv, c);
        int m = grid_candidates_buf(&g, c, &cand, &ccap);
        if (m < 0) {
            free(cand);
            grid_free(&g);
            return -1;
        }
        for (int k = 0; k < m; ++k) {
            int j = cand[k];
            float rx = bpos3[3 * b] - x3[3 * j];
            float ry = bpos3[3 * b + 1] - x3[3 * j + 1];
            float rz = bpos3[3 * b + 2] - x3[3 * j + 2];
            float r_sq = sqn3(rx, ry, rz);
            if (r_sq >= hh) continue;
            float rho_f = (rho[j] < 1.0f) ? 1.0f : rho[j]; /* std::max(rho, 1.0f) */
            float pd = rho_f - rho0;
            float pressure = (0.0f < pd) ? pd : 0.0f; /* std::max(0.0f, rho_f - rho0) */
            float pressure_coeff = mass * pressure / (rho_f * rho_f);
            float gr[3];
            spiky_grad3(rx, ry, rz, h, &gr[0], &gr[1], &gr[2]);
            float a = pressure_coeff * rho0 * psi_b;
            f[0] += a * gr[0];
            f[1] += a * gr[1];
            f[2] += a * gr[2];
        }
        if (sqn3(f[0], f[1], f[2]) > 1e-20f) {
            force3[3 * bi] += f[0];
            force3[3 * bi + 1] += f[1];
            force3[3 * bi + 2] += f[2];
            float ra0 = bpos3[3 * b] - body_pos3[3 * bi];
            float ra1 = bpos3[3 * b + 1] - body_pos3[3 * bi + 1];
            float ra2 = bpos3[3 * b + 2] - body_pos3[3 * bi + 2];
            torque3[3 * bi] += ra1 * f[2] - ra2 * f[1];
            torque3[3 * bi + 1] += ra2 * f[0] - ra0 * f[2];
            torque3[3 * bi + 2] += ra0 * f[1] - ra1 * f[0];
        }
    }
    free(cand);
    grid_free(&g);
    return 0;
}

int orc_sample_box(const float* he, const float* lt_pos, const float* lt_quat, float spacing,
                   float* out3, int cap) {
    /* boundary.cpp:15-53 */
    int m = 0;
    for (int axis = 0; axis < 3; ++axis) {
        int a1 = (axis + 1) % 3;
        int a2 = (axis + 2) % 3;
        int n1 = (int)floorf(2.0f * he[a1] / spacing) + 1;
        int n2 = (int)floorf(2.0f * he[a2] / spacing) + 1;
        if (n1 < 1) n1 = 1;
        if (n2 < 1) n2 = 1;
        for (int sign = -1; sign <= 1; sign += 2)
            for (int i1 = 0; i1 < n1; ++i1)
                for (int i2 = 0; i2 < n2; ++i2) {
                    float lp[3] = {0.0f, 0.0f, 0.0f};
                    lp[axis] = (float)sign * he[axis];
                    lp[a1] = -he[a1] + (float)i1 * spacing;
                    lp[a2] = -he[a2] + (float)i2 * spacing;
                    if (m < cap) transform_point(lt_pos, lt_quat, lp, out3 + 3 * m);
                    ++m;
                }
    }
    return m;
}

int orc_sample_sphere(float r, const float* lt_pos, const float* lt_quat, float spacing,
                      float* out3, int cap) {
    /* boundary.cpp:55-91 */
    const float pi = 3.14159265358979323846f; /* std::numbers::pi_v<float> */
    const float area = 4.0f * pi * r * r;
    int n = (int)(area / (spacing * spacing));
    if (n < 12) n = 12;
    const float golden_ratio = (1.0f + sqrtf(5.0f)) / 2.0f;
    const float golden_angle = 2.0f * pi / (golden_ratio * golden_ratio);
    for (int i = 0; i < n; ++i) {
        float theta = acosf(1.0f - 2.0f * ((float)i + 0.5f) / (float)n);
        float phi = golden_angle * (float)i;
        float lp[3] = {r * sinf(theta) * cosf(phi), r * sinf(theta) * sinf(phi), r * cosf(theta)};
        if (i < cap) transform_point(lt_pos, lt_quat, lp, out3 + 3 * i);
    }
    return n;
}

static void normalized3(float* a) {
    float z = sqn3(a[0], a[1], a[2]);
    if (z > 0.0f) {
        float s = sqrtf(z);
        a[0] = a[0] / s;
        a[1] = a[1] / s;
        a[2] = a[2] / s;
    }
}

static void cross3(const float* a, const float* b, float* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

int orc_sample_plane(const float* normal, float offset, float spacing, float extent, float* out3,
                     int cap) {
    /* boundary.cpp:93-126 */
    float t1[3], t2[3];
    if (fabsf(normal[1]) < 0.9f) {
        const float ey[3] = {0.0f, 1.0f, 0.0f};
        cross3(ey, normal, t1);
    } else {
        const float ex[3] = {1.0f, 0.0f, 0.0f};
        cross3(ex, normal, t1);
    }
    normalized3(t1);
    cross3(normal, t1, t2);
    normalized3(t2);
    int n = (int)floorf(2.0f * extent / spacing) + 1;
    int m = 0;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            float s = -extent + (float)i * spacing;
            float t = -extent + (float)j * spacing;
            if (m < cap)
                for (int c = 0; c < 3; ++c)
                    out3[3 * m + c] = (normal[c] * offset + t1[c] * s) + t2[c] * t;
            ++m;
        }
    return m;
}

int orc_generate_block(const float* lower, const float* upper, float spacing, float* out3,
                       int cap) {
    /* particle_state.cpp:31-58 */
    if (spacing <= 0.0f) return 0;
    int nx = (int)floorf((upper[0] - lower[0]) / spacing) + 1;
    int ny = (int)floorf((upper[1] - lower[1]) / spacing) + 1;
    int nz = (int)floorf((upper[2] - lower[2]) / spacing) + 1;
    if (nx < 1) nx = 1;
    if (ny < 1) ny = 1;
    if (nz < 1) nz = 1;
    int m = 0;
    for (int iz = 0; iz < nz; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix) {
                if (m < cap) {
                    out3[3 * m] = lower[0] + (float)ix * spacing;
                    out3[3 * m + 1] = lower[1] + (float)iy * spacing;
                    out3[3 * m + 2] = lower[2] + (float)iz * spacing;
                }
                ++m;
            }
    return m;
}
