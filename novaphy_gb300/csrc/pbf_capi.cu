// C ABI of the PBF step (include/novaphy_pbf.h): scene lifetime, host<->device
// transfer, settings -> per-step constants, and step orchestration with CUDA
// graph replay.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "novaphy_pbf.h"
#include "pbf_boundary.cuh"
#include "pbf_internal.cuh"
#include "pbf_launch.cuh"
#include "pbf_types.cuh"
#include "radix_sort.cuh"

using namespace pbf;

namespace {

thread_local std::string g_last_error;

constexpr float kPi = 3.14159265358979323846f;  // math_utils.h:53

}  // namespace

namespace pbf {
namespace capi {

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* where) {
    const int code = (e == cudaErrorMemoryAllocation) ? PBF_ERR_OOM
                     : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
                         ? PBF_ERR_NO_DEVICE
                         : PBF_ERR_CUDA;
    return fail(code, std::string(where) + ": " + cudaGetErrorString(e));
}

}  // namespace capi
}  // namespace pbf

using namespace pbf::capi;

namespace {

__global__ void k_expand3(const float* __restrict__ a3, float4* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_float4(a3[3 * i], a3[3 * i + 1], a3[3 * i + 2], 0.0f);
}

__global__ void k_pack3(const float4* __restrict__ in, float* __restrict__ a3, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const float4 t = in[i];
        a3[3 * i] = t.x;
        a3[3 * i + 1] = t.y;
        a3[3 * i + 2] = t.z;
    }
}

__global__ void k_finite(const float4* __restrict__ x, const float4* __restrict__ v, int n,
                         uint32_t* __restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const float4 a = x[i], b = v[i];
        if (!(isfinite(a.x) && isfinite(a.y) && isfinite(a.z) && isfinite(b.x) && isfinite(b.y) &&
              isfinite(b.z)))
            atomicOr(flag, 1u);
    }
}

}  // namespace

namespace pbf {
// Sets the calling thread's pbf_last_error() text (used by other translation
// units of the library).
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace pbf

namespace pbf {
namespace capi {

// One stream-ordered memory pool per device for scene state and scratch.
// Freed blocks stay in the pool (release threshold: never), so opening and
// closing scenes neither synchronizes the device, as cudaMalloc/cudaFree
// would, nor hands memory back to the driver between scenes.
cudaMemPool_t scene_pool(int device) {
    static std::mutex mu;
    static std::vector<cudaMemPool_t> pools;
    std::lock_guard<std::mutex> lk(mu);
    if ((int)pools.size() <= device) pools.resize((size_t)device + 1, nullptr);
    if (!pools[device]) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        cudaMemPool_t pool = nullptr;
        if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) return nullptr;
        unsigned long long keep = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        pools[device] = pool;
    }
    return pools[device];
}

int pool_alloc(void** p, size_t bytes, int device, cudaStream_t st) {
    cudaMemPool_t pool = scene_pool(device);
    if (!pool) return fail(PBF_ERR_CUDA, "cudaMemPoolCreate failed");
    PBF_CUDA(cudaMallocFromPoolAsync(p, bytes, pool, st));
    return PBF_OK;
}

void pool_free(void* p, cudaStream_t st) {
    if (p) cudaFreeAsync(p, st);
}

}  // namespace capi
}  // namespace pbf

namespace {

void free_particles(pbf_scene* s) {
    ++s->buf_gen;
    if (s->graph) {
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    for (void* m : {s->pmem, s->wmem, s->smem}) pool_free(m, s->stream);
    s->pmem = s->wmem = s->smem = nullptr;
    s->cap = s->work_cap = 0;
    s->sort = SortScratch{};
    s->B = StepBuffers{};
    s->B.off = s->off;
    if (s->off) {
        s->B.slot_alias = reinterpret_cast<unsigned char*>(s->off) +
                          align_up((size_t)s->off_cap * 4, 256);
        s->B.moved = reinterpret_cast<uint32_t*>(s->B.slot_alias + align_up(s->off_cap, 256));
        s->B.lamnz = s->B.moved + s->off_cap;
        s->B.dhist = s->B.lamnz + s->off_cap;
    }
}

// (Re)allocates the resident state for `cap` particles; the step scratch
// follows on the next step (ensure_work).
int alloc_particles(pbf_scene* s, int cap) {
    free_particles(s);
    const int c = cap > 0 ? cap : 1;
    const size_t f4 = align_up((size_t)c * 16, 256);
    const size_t f1 = align_up((size_t)c * 4, 256);
    const size_t f3 = align_up((size_t)c * 12, 256);
    const size_t total = 2 * f4 + 2 * f1 + f3;
    int rc = pool_alloc(&s->pmem, total, s->device, s->stream);
    if (rc) return rc;
    char* p = reinterpret_cast<char*>(s->pmem);
    s->B.x = reinterpret_cast<float4*>(p);
    s->B.v = reinterpret_cast<float4*>(p + f4);
    s->B.rho = reinterpret_cast<float*>(p + 2 * f4);
    s->B.lam = reinterpret_cast<float*>(p + 2 * f4 + f1);
    s->staging = reinterpret_cast<float*>(p + 2 * f4 + 2 * f1);
    PBF_CUDA(cudaMemsetAsync(s->pmem, 0, total, s->stream));
    s->cap = c;
    return PBF_OK;
}

// Step scratch for the scene's capacity (sorted copies, keys, buckets, sort).
int ensure_work(pbf_scene* s) {
    if (s->wmem && s->work_cap >= s->cap) return PBF_OK;
    ++s->buf_gen;
    if (s->graph) {
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    for (void* m : {s->wmem, s->smem}) pool_free(m, s->stream);
    s->wmem = s->smem = nullptr;
    s->work_cap = 0;
    const int c = s->cap > 0 ? s->cap : 1;
    // The step scratch batches share, then the scene's run ends.
    const size_t wb = work_bytes(c) + align_up((size_t)c * 4, 256);
    int rc = pool_alloc(&s->wmem, wb, s->device, s->stream);
    if (rc) return rc;
    PBF_CUDA(cudaMemsetAsync(s->wmem, 0, wb, s->stream));
    bind_work(s->B, s->wmem, c);
    s->B.segend = reinterpret_cast<uint32_t*>(static_cast<char*>(s->wmem) + work_bytes(c));
    const size_t sb = sort_scratch_bytes(c);
    rc = pool_alloc(&s->smem, sb, s->device, s->stream);
    if (rc) return rc;
    PBF_CUDA(cudaMemsetAsync(s->smem, 0, sb, s->stream));
    sort_scratch_bind(s->sort, s->smem, c);
    s->B.err = s->sort.err;
    s->work_cap = c;
    return PBF_OK;
}

}  // namespace

namespace pbf {
namespace capi {

int check_settings(const pbf_settings* st) {
    if (!st) return fail(PBF_ERR_INVALID_ARG, "settings is NULL");
    if (!(st->kernel_radius > 0.0f) || !std::isfinite(st->kernel_radius))
        return fail(PBF_ERR_INVALID_ARG, "kernel_radius must be a positive finite number");
    if (!(st->rest_density > 0.0f))
        return fail(PBF_ERR_INVALID_ARG, "rest_density must be positive");
    if (st->solver_iterations < 0 || st->solver_iterations > 1000)
        return fail(PBF_ERR_INVALID_ARG, "solver_iterations must be in [0, 1000]");
    return PBF_OK;
}

// Grid fitted to the domain (clamp on, two cells of margin) or to the
// particles' bounding box (clamp off).  Without the clamp nothing keeps the
// fluid inside its first box, so that grid gets max(8, extent) cells of
// margin per side, up to 256: a resident scene whose fluid falls or spreads
// keeps its particles in the grid for many steps instead of wrapping onto the
// slower aliased-bucket walk (any fit gives the same results).  Each axis
// >= 4 and at most 2^24 slots in total.
GridDesc fit_grid(const pbf_scene* s) {
    const pbf_settings& st = s->settings;
    const float inv = 1.0f / st.kernel_radius;
    float lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
        if (st.use_domain_bounds) {
            lo[d] = std::min(st.domain_lower[d], st.domain_upper[d]);
            hi[d] = std::max(st.domain_lower[d], st.domain_upper[d]);
        } else if (s->have_bbox) {
            lo[d] = s->bbox_lo[d];
            hi[d] = s->bbox_hi[d];
        } else {
            lo[d] = 0.0f;
            hi[d] = 0.0f;
        }
    }
    const long long kMaxSlots = 1LL << 24;
    long long a0[3], ext[3], mar[3];
    for (int d = 0; d < 3; ++d) {
        double a = std::floor((double)lo[d] * inv), b = std::floor((double)hi[d] * inv);
        if (!std::isfinite(a) || !std::isfinite(b) || b - a > 4096.0) b = a + 4096.0;
        if (!std::isfinite(a) || std::fabs(a) > 1e9) a = 0.0, b = 4096.0;
        a0[d] = (long long)a;
        ext[d] = (long long)(b - a);
        mar[d] = st.use_domain_bounds ? 2 : std::min<long long>(256, std::max<long long>(8, ext[d]));
    }
    // The margin gives way first when the slots would exceed the cap.
    auto slots = [&](long long cap_m) {
        long long p = 1;
        for (int d = 0; d < 3; ++d) p *= std::max(4LL, ext[d] + 2 * std::min(mar[d], cap_m) + 1);
        return p;
    };
    long long cap_m = 256;
    while (cap_m > 2 && slots(cap_m) > kMaxSlots) cap_m /= 2;
    long long o[3], g[3];
    for (int d = 0; d < 3; ++d) {
        const long long m = std::max(2LL, std::min(mar[d], cap_m));
        o[d] = a0[d] - m;
        g[d] = std::max(4LL, ext[d] + 2 * m + 1);
    }
    while (g[0] * g[1] * g[2] > kMaxSlots) {
        int m = 0;
        for (int d = 1; d < 3; ++d)
            if (g[d] > g[m]) m = d;
        g[m] = std::max(4LL, g[m] / 2);
    }
    GridDesc G{};
    G.ox = (int)o[0];
    G.oy = (int)o[1];
    G.oz = (int)o[2];
    G.gx = (int)g[0];
    G.gy = (int)g[1];
    G.gz = (int)g[2];
    G.nslots = (uint32_t)(g[0] * g[1] * g[2]);
    int bits = 1;
    while ((1ull << bits) < (unsigned long long)G.nslots) ++bits;
    G.key_bits = bits;
    return G;
}

}  // namespace capi
}  // namespace pbf

namespace {

int ensure_offsets(pbf_scene* s, uint32_t nslots) {
    if (s->off && s->off_cap >= nslots + 1) return PBF_OK;
    ++s->buf_gen;
    if (s->graph) {
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    if (s->off) cudaFree(s->off);
    s->off = nullptr;
    // offsets (nslots + 1 words), one alias byte per slot, a moved word and
    // a lambda word per slot, then the density pass's walk counts
    const size_t ob = align_up((size_t)(nslots + 1) * 4, 256);
    const size_t ab = align_up(nslots + 1, 256);
    PBF_CUDA(cudaMalloc(&s->off, ob + ab + (size_t)(nslots + 1) * 8 + 4 * kWalkHist * 4));
    s->off_cap = nslots + 1;
    s->B.off = s->off;
    s->B.slot_alias = reinterpret_cast<unsigned char*>(s->off) + ob;
    s->B.moved = reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(s->off) + ob + ab);
    s->B.lamnz = s->B.moved + (nslots + 1);
    s->B.dhist = s->B.lamnz + (nslots + 1);
    PBF_CUDA(cudaMemsetAsync(s->B.dhist, 0, 4 * kWalkHist * 4, s->stream));
    return PBF_OK;
}

float host_poly6(float r_sq, float h) {
    // sph_kernel.h:24-30, float arithmetic, no contraction.
    if (r_sq >= h * h) return 0.0f;
    float h2 = h * h;
    float diff = h2 - r_sq;
    float h9 = h2 * h2 * h2 * h2 * h;
    return (315.0f / (64.0f * kPi * h9)) * diff * diff * diff;
}

}  // namespace

namespace pbf {
namespace capi {

// Per-step constants from settings (operation order of pbf_solver.cpp).
int scene_consts(const pbf_scene* s, float dt, StepConsts& C) {
    const pbf_settings& st = s->settings;
    if (!(dt > 0.0f) || !std::isfinite(dt)) return fail(PBF_ERR_INVALID_ARG, "dt must be > 0");
    std::memset(&C, 0, sizeof(C));
    C.n = s->n;
    const float h = st.kernel_radius;
    C.h = h;
    C.h2 = h * h;
    {
        // Smallest float g with sqrtf(g) >= h; any r_sq >= max(h2, g) gives
        // poly6 == 0 and spiky_grad == 0 (sph_kernel.h:25, :40).
        float g = C.h2;
        if (std::sqrt(g) >= h) {
            for (int k = 0; k < 64; ++k) {
                float p = std::nextafter(g, 0.0f);
                if (std::sqrt(p) >= h) g = p;
                else break;
            }
        } else {
            for (int k = 0; k < 64 && std::sqrt(g) < h; ++k) g = std::nextafter(g, INFINITY);
        }
        C.cut = std::max(C.h2, g);
    }
    C.inv_cell = 1.0f / h;
    C.mass = s->mass;
    C.rho0 = st.rest_density;
    C.inv_rho0 = 1.0f / st.rest_density;
    C.eps = st.epsilon;
    C.mr = s->mass * C.inv_rho0;
    {
        float h2 = h * h;
        float h9 = h2 * h2 * h2 * h2 * h;
        C.k_poly = 315.0f / (64.0f * kPi * h9);
        float h6 = h * h * h * h * h * h;
        C.k_spiky = -(45.0f / (kPi * h6));
    }
    const float delta_q = st.corr_delta_q * h;
    C.w_dq = host_poly6(delta_q * delta_q, h);
    C.neg_corr_k = -st.corr_k;
    C.corr_n4 = st.corr_n == 4 ? 1 : 0;
    C.scorr_on = C.w_dq > 1e-10f ? 1 : 0;
    C.dt = dt;
    C.inv_dt = 1.0f / dt;
    C.max_speed = h / dt;
    C.max_speed_sq = C.max_speed * C.max_speed;
    for (int d = 0; d < 3; ++d) C.g[d] = s->gravity[d];
    C.xsph_c = st.xsph_viscosity;
    C.xsph_on = st.xsph_viscosity > 0.0f ? 1 : 0;
    C.vort_eps = st.vorticity_epsilon;
    C.vort_scale = dt * st.vorticity_epsilon;
    C.vort_on = st.vorticity_epsilon > 0.0f ? 1 : 0;
    C.clamp = st.use_domain_bounds ? 1 : 0;
    const float pr = st.particle_radius;
    for (int d = 0; d < 3; ++d) {
        C.lo[d] = st.domain_lower[d] + pr;
        C.hi[d] = st.domain_upper[d] - pr;
    }
    C.hash_compat = st.hash_compat ? 1 : 0;
    C.two_way = st.boundary_two_way ? 1 : 0;
    C.bfric = st.boundary_two_way ? st.boundary_friction : 0.0f;
    C.iters = st.solver_iterations;
    C.seg_begin = 0;
    C.seg_end = (uint32_t)s->n;
    C.grid = fit_grid(s);
    return PBF_OK;
}

}  // namespace capi
}  // namespace pbf

namespace {

// Constants of the scene's own step, with its offsets table and scratch.
int make_consts(pbf_scene* s, float dt, StepConsts& C) {
    int rc = scene_consts(s, dt, C);
    if (!rc) rc = ensure_offsets(s, C.grid.nslots);
    if (!rc) rc = ensure_work(s);
    return rc;
}

void update_bbox(pbf_scene* s, const float* x3, int n) {
    if (n <= 0 || !x3) {
        s->have_bbox = false;
        return;
    }
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            const float t = x3[3 * i + d];
            if (std::isfinite(t)) {
                lo[d] = std::min(lo[d], t);
                hi[d] = std::max(hi[d], t);
            }
        }
    for (int d = 0; d < 3; ++d) {
        if (!(lo[d] <= hi[d])) lo[d] = hi[d] = 0.0f;
        // Leave room for the fluid to spread.
        const float ext = hi[d] - lo[d];
        s->bbox_lo[d] = lo[d] - 0.5f * ext;
        s->bbox_hi[d] = hi[d] + 0.5f * ext;
    }
    s->have_bbox = true;
}

int upload3(pbf_scene* s, const float* host3, float4* dst, int n) {
    if (n <= 0) return PBF_OK;
    PBF_CUDA(cudaMemcpyAsync(s->staging, host3, (size_t)n * 12, cudaMemcpyHostToDevice, s->stream));
    k_expand3<<<(n + 255) / 256, 256, 0, s->stream>>>(s->staging, dst, n);
    PBF_CUDA(cudaGetLastError());
    return PBF_OK;
}

int download3(pbf_scene* s, const float4* src, float* host3, int n) {
    if (n <= 0) return PBF_OK;
    k_pack3<<<(n + 255) / 256, 256, 0, s->stream>>>(src, s->staging, n);
    PBF_CUDA(cudaGetLastError());
    PBF_CUDA(cudaMemcpyAsync(host3, s->staging, (size_t)n * 12, cudaMemcpyDeviceToHost, s->stream));
    return PBF_OK;
}

int set_state(pbf_scene* s, int n, const float* x3, const float* v3) {
    if (n < 0) return fail(PBF_ERR_INVALID_ARG, "n must be >= 0");
    if (n > 0 && !x3) return fail(PBF_ERR_INVALID_ARG, "positions are NULL");
    if (n > (1 << 29)) return fail(PBF_ERR_CAPACITY, "at most 2^29 particles per scene");
    if (n > s->cap || !s->pmem) {
        int rc = alloc_particles(s, n);
        if (rc) return rc;
    }
    s->n = n;
    if (n == 0) return PBF_OK;
    int rc = upload3(s, x3, s->B.x, n);
    if (rc) return rc;
    if (v3) {
        rc = upload3(s, v3, s->B.v, n);
        if (rc) return rc;
    } else {
        PBF_CUDA(cudaMemsetAsync(s->B.v, 0, (size_t)n * 16, s->stream));
    }
    PBF_CUDA(cudaMemsetAsync(s->B.rho, 0, (size_t)n * 4, s->stream));
    PBF_CUDA(cudaMemsetAsync(s->B.lam, 0, (size_t)n * 4, s->stream));
    // The grid follows the domain when the clamp is on; otherwise it is
    // fitted to the particles given here.
    if (!s->settings.use_domain_bounds) update_bbox(s, x3, n);
    return PBF_OK;
}

bool consts_equal(const StepConsts& a, const StepConsts& b) {
    return std::memcmp(&a, &b, sizeof(StepConsts)) == 0;
}

int enqueue(pbf_scene* s, const StepConsts& C, cudaStream_t st, PhaseMarks* pm = nullptr) {
    const int iters = s->settings.solver_iterations;
    cudaError_t e = s->settings.exact_arithmetic
                        ? exact_enqueue_step(s->B, C, iters, s->sort, st, pm)
                        : fast_enqueue_step(s->B, C, iters, s->sort, st, pm);
    if (e != cudaSuccess) return cuda_fail(e, "enqueue_step");
    return PBF_OK;
}

bool graphs_enabled() {
    const char* v = std::getenv("PBF_NO_GRAPH");
    return !(v && v[0] == '1');
}

int run_steps(pbf_scene* s, float dt, int nsteps) {
    if (nsteps < 0) return fail(PBF_ERR_INVALID_ARG, "nsteps must be >= 0");
    if (s->n == 0 || nsteps == 0) return PBF_OK;  // pbf_solver.cpp:21
    StepConsts C;
    int rc = make_consts(s, dt, C);
    if (rc) return rc;
    if (!graphs_enabled()) {
        for (int k = 0; k < nsteps; ++k) {
            rc = enqueue(s, C, s->stream);
            if (rc) return rc;
        }
        return PBF_OK;
    }
    const int iters = s->settings.solver_iterations;
    const int exact = s->settings.exact_arithmetic ? 1 : 0;
    if (!s->graph || !consts_equal(C, s->graph_consts) || iters != s->graph_iters ||
        exact != s->graph_exact) {
        if (s->graph) {
            cudaGraphExecDestroy(s->graph);
            s->graph = nullptr;
        }
        cudaGraph_t g = nullptr;
        PBF_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        const int erc = enqueue(s, C, s->stream);
        cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
        if (erc) {
            if (g) cudaGraphDestroy(g);
            return erc;
        }
        if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
        ce = cudaGraphInstantiate(&s->graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            s->graph = nullptr;
            return cuda_fail(ce, "cudaGraphInstantiate");
        }
        s->graph_consts = C;
        s->graph_iters = iters;
        s->graph_exact = exact;
    }
    for (int k = 0; k < nsteps; ++k) PBF_CUDA(cudaGraphLaunch(s->graph, s->stream));
    return PBF_OK;
}

int sync_and_check(pbf_scene* s) {
    PBF_CUDA(cudaStreamSynchronize(s->stream));
    if (!s->sort.err) return PBF_OK;
    uint32_t err = 0;
    PBF_CUDA(cudaMemcpy(&err, s->sort.err, 4, cudaMemcpyDeviceToHost));
    if (err) {
        PBF_CUDA(cudaMemset(s->sort.err, 0, 4));
        return fail(PBF_ERR_TIMEOUT, "device-side wait in the cell sort gave up (error word " +
                                         std::to_string(err) + ")");
    }
    return PBF_OK;
}

}  // namespace

// ---------------------------------------------------------------------------

extern "C" {

const char* pbf_version(void) { return "novaphy_gb300 pbf 1 (sm_103a)"; }

const char* pbf_last_error(void) { return g_last_error.c_str(); }

int pbf_default_settings(pbf_settings* out) {
    if (!out) return fail(PBF_ERR_INVALID_ARG, "out is NULL");
    pbf_settings d{};
    // PBFSettings defaults, include/novaphy/fluid/pbf_solver.h:14-27.
    d.rest_density = 1000.0f;
    d.kernel_radius = 0.1f;
    d.particle_radius = 0.025f;
    d.solver_iterations = 4;
    d.epsilon = 100.0f;
    d.xsph_viscosity = 0.01f;
    d.vorticity_epsilon = 0.0f;
    d.corr_delta_q = 0.3f;
    d.corr_k = 0.001f;
    d.corr_n = 4;
    d.use_domain_bounds = 0;
    d.domain_lower[0] = -10.0f;
    d.domain_lower[1] = 0.0f;
    d.domain_lower[2] = -10.0f;
    d.domain_upper[0] = 10.0f;
    d.domain_upper[1] = 10.0f;
    d.domain_upper[2] = 10.0f;
    d.exact_arithmetic = 1;
    d.hash_compat = 1;
    d.boundary_two_way = 0;
    d.boundary_friction = 0.0f;
    *out = d;
    return PBF_OK;
}

int pbf_device_count(int* out) {
    if (!out) return fail(PBF_ERR_INVALID_ARG, "out is NULL");
    int c = 0;
    cudaError_t e = cudaGetDeviceCount(&c);
    if (e != cudaSuccess) {
        *out = 0;
        return cuda_fail(e, "cudaGetDeviceCount");
    }
    *out = c;
    return PBF_OK;
}

int pbf_scene_create(int device, const pbf_settings* settings, int n, const float* x3,
                     const float* v3, float mass, pbf_scene** out) {
    if (!out) return fail(PBF_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    int rc = check_settings(settings);
    if (rc) return rc;
    int count = 0;
    cudaError_t ce = cudaGetDeviceCount(&count);
    if (ce != cudaSuccess || count == 0)
        return fail(PBF_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(ce));
    if (device < 0 || device >= count) return fail(PBF_ERR_INVALID_ARG, "device out of range");
    DeviceGuard dg(device);
    if (!dg.ok) return fail(PBF_ERR_NO_DEVICE, "cudaSetDevice failed");
    pbf_scene* s = new pbf_scene();
    s->device = device;
    s->settings = *settings;
    s->mass = mass;
    ce = cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) {
        delete s;
        return cuda_fail(ce, "cudaStreamCreate");
    }
    s->stream = s->own_stream;
    rc = set_state(s, n, x3, v3);
    if (rc == PBF_OK) {
        ce = cudaStreamSynchronize(s->stream);
        if (ce != cudaSuccess) rc = cuda_fail(ce, "cudaStreamSynchronize");
    }
    if (rc) {
        pbf_scene_destroy(s);
        return rc;
    }
    *out = s;
    return PBF_OK;
}

int pbf_scene_destroy(pbf_scene* s) {
    if (!s) return PBF_OK;
    {
        DeviceGuard dg(s->device);
        if (s->stream) cudaStreamSynchronize(s->stream);
        for (void* m : {s->bnd.mem, s->bnd.body_mem, s->bnd.sort_mem, s->bnd.fq_mem,
                        s->bnd.tw_mem, static_cast<void*>(s->bnd.rb),
                        static_cast<void*>(s->bnd.shapes)})
            if (m) cudaFree(m);
        if (s->bnd.idx.off) cudaFree(s->bnd.idx.off);
        if (s->couple_graph) cudaGraphExecDestroy(s->couple_graph);
        free_particles(s);
        if (s->off) cudaFree(s->off);
        if (s->d_flag) cudaFree(s->d_flag);
        if (s->ev) cudaEventDestroy(s->ev);
        if (s->own_stream) {
            cudaStreamSynchronize(s->own_stream);
            cudaStreamDestroy(s->own_stream);
        }
    }
    delete s;
    return PBF_OK;
}

int pbf_scene_set_settings(pbf_scene* s, const pbf_settings* settings) {
    if (!s) return fail(PBF_ERR_INVALID_ARG, "scene is NULL");
    int rc = check_settings(settings);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(s->mu);
    s->settings = *settings;
    return PBF_OK;
}

int pbf_scene_get_settings(const pbf_scene* s, pbf_settings* out) {
    if (!s || !out) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    *out = s->settings;
    return PBF_OK;
}

int pbf_scene_set_gravity(pbf_scene* s, const float* g3) {
    if (!s || !g3) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    for (int d = 0; d < 3; ++d) s->gravity[d] = g3[d];
    return PBF_OK;
}

int pbf_scene_set_mass(pbf_scene* s, float mass) {
    if (!s) return fail(PBF_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    s->mass = mass;
    return PBF_OK;
}

int pbf_scene_num_particles(const pbf_scene* s, int* out) {
    if (!s || !out) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    *out = s->n;
    return PBF_OK;
}

int pbf_scene_reset(pbf_scene* s, int n, const float* x3, const float* v3) {
    if (!s) return fail(PBF_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    int rc = set_state(s, n, x3, v3);
    if (rc) return rc;
    PBF_CUDA(cudaStreamSynchronize(s->stream));
    return PBF_OK;
}

int pbf_scene_step(pbf_scene* s, float dt, int nsteps) {
    if (!s) return fail(PBF_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    return run_steps(s, dt, nsteps);
}

int pbf_scene_step_timed(pbf_scene* s, float dt, int nsteps, float* ms_out) {
    if (!s || !ms_out) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    *ms_out = 0.0f;
    cudaEvent_t a = nullptr, b = nullptr;
    PBF_CUDA(cudaEventCreate(&a));
    cudaError_t e = cudaEventCreate(&b);
    int rc = PBF_OK;
    if (e == cudaSuccess) e = cudaEventRecord(a, s->stream);
    if (e == cudaSuccess) rc = run_steps(s, dt, nsteps);
    if (e == cudaSuccess && rc == PBF_OK) e = cudaEventRecord(b, s->stream);
    if (e == cudaSuccess && rc == PBF_OK) e = cudaEventSynchronize(b);
    if (e == cudaSuccess && rc == PBF_OK) e = cudaEventElapsedTime(ms_out, a, b);
    cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "pbf_scene_step_timed");
    return sync_and_check(s);
}

}  // extern "C"

namespace {
size_t snapshot_bytes(int n) { return (size_t)n * (16 + 16 + 4 + 4); }
}  // namespace

extern "C" {

int pbf_snapshot_create(pbf_scene* s, pbf_snapshot** out) {
    if (!s || !out) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    pbf_snapshot* snap = new pbf_snapshot();
    snap->device = s->device;
    snap->n = s->n;
    snap->settings = s->settings;
    for (int d = 0; d < 3; ++d) snap->gravity[d] = s->gravity[d];
    snap->mass = s->mass;
    if (s->n > 0) {
        cudaError_t e = cudaMalloc(&snap->mem, snapshot_bytes(s->n));
        if (e != cudaSuccess) {
            delete snap;
            return cuda_fail(e, "pbf_snapshot_create");
        }
        char* p = reinterpret_cast<char*>(snap->mem);
        const size_t n = (size_t)s->n;
        e = cudaMemcpyAsync(p, s->B.x, n * 16, cudaMemcpyDeviceToDevice, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(p + n * 16, s->B.v, n * 16, cudaMemcpyDeviceToDevice, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(p + n * 32, s->B.rho, n * 4, cudaMemcpyDeviceToDevice, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(p + n * 36, s->B.lam, n * 4, cudaMemcpyDeviceToDevice, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) {
            cudaFree(snap->mem);
            delete snap;
            return cuda_fail(e, "pbf_snapshot_create");
        }
    }
    *out = snap;
    return PBF_OK;
}

int pbf_snapshot_destroy(pbf_snapshot* snap) {
    if (!snap) return PBF_OK;
    if (snap->mem) {
        DeviceGuard dg(snap->device);
        cudaFree(snap->mem);
    }
    delete snap;
    return PBF_OK;
}

int pbf_snapshot_num_particles(const pbf_snapshot* snap, int* out) {
    if (!snap || !out) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    *out = snap->n;
    return PBF_OK;
}

}  // extern "C"

namespace pbf {
namespace capi {

int restore_on(pbf_scene* s, const pbf_snapshot* snap, cudaStream_t st) {
    if (snap->device != s->device) return fail(PBF_ERR_INVALID_ARG, "snapshot is on another device");
    if (snap->n > s->cap || !s->pmem) {
        int rc = alloc_particles(s, snap->n);
        if (rc) return rc;
    }
    s->n = snap->n;
    s->settings = snap->settings;
    for (int d = 0; d < 3; ++d) s->gravity[d] = snap->gravity[d];
    s->mass = snap->mass;
    if (snap->n == 0) return PBF_OK;
    const char* p = reinterpret_cast<const char*>(snap->mem);
    const size_t n = (size_t)snap->n;
    PBF_CUDA(cudaMemcpyAsync(s->B.x, p, n * 16, cudaMemcpyDeviceToDevice, st));
    PBF_CUDA(cudaMemcpyAsync(s->B.v, p + n * 16, n * 16, cudaMemcpyDeviceToDevice, st));
    PBF_CUDA(cudaMemcpyAsync(s->B.rho, p + n * 32, n * 4, cudaMemcpyDeviceToDevice, st));
    PBF_CUDA(cudaMemcpyAsync(s->B.lam, p + n * 36, n * 4, cudaMemcpyDeviceToDevice, st));
    return PBF_OK;
}

uint32_t grid_slots_for(const pbf_settings& st, const float* x3, int n) {
    pbf_scene tmp;
    tmp.settings = st;
    if (!st.use_domain_bounds) update_bbox(&tmp, x3, n);
    return fit_grid(&tmp).nslots;
}

size_t scene_device_bytes(const pbf_scene* s) {
    size_t b = 0;
    if (s->pmem) {
        const int c = s->cap > 0 ? s->cap : 1;
        b += 2 * align_up((size_t)c * 16, 256) + 2 * align_up((size_t)c * 4, 256) +
             align_up((size_t)c * 12, 256);
    }
    if (s->wmem)
        b += work_bytes(s->work_cap) + align_up((size_t)s->work_cap * 4, 256) +
             sort_scratch_bytes(s->work_cap);
    if (s->off)
        b += align_up((size_t)s->off_cap * 4, 256) + align_up(s->off_cap, 256) +
             (size_t)s->off_cap * 8 + 4 * kWalkHist * 4;
    return b;
}

}  // namespace capi
}  // namespace pbf

namespace {
// Copies a snapshot into the scene on its stream (asynchronous).
int restore_async(pbf_scene* s, const pbf_snapshot* snap) { return restore_on(s, snap, s->stream); }
}  // namespace

extern "C" {

int pbf_snapshot_restore(pbf_scene* s, const pbf_snapshot* snap) {
    if (!s || !snap) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    int rc = restore_async(s, snap);
    if (rc) return rc;
    PBF_CUDA(cudaStreamSynchronize(s->stream));
    return PBF_OK;
}

int pbf_scene_replay_timed(pbf_scene* s, const pbf_snapshot* seed, float dt, int nsteps,
                           float* ms_out) {
    if (!s || !seed || !ms_out) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    if (nsteps < 0) return fail(PBF_ERR_INVALID_ARG, "nsteps must be >= 0");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    *ms_out = 0.0f;
    int rc = restore_async(s, seed);
    if (rc) return rc;
    rc = run_steps(s, dt, 1);  // capture the step graph outside the timed region
    if (rc) return rc;
    cudaEvent_t a = nullptr, b = nullptr;
    PBF_CUDA(cudaEventCreate(&a));
    cudaError_t e = cudaEventCreate(&b);
    if (e == cudaSuccess) e = cudaEventRecord(a, s->stream);
    for (int k = 0; k < nsteps && e == cudaSuccess && rc == PBF_OK; ++k) {
        rc = restore_async(s, seed);
        if (rc == PBF_OK) rc = run_steps(s, dt, 1);
    }
    if (e == cudaSuccess && rc == PBF_OK) e = cudaEventRecord(b, s->stream);
    if (e == cudaSuccess && rc == PBF_OK) e = cudaEventSynchronize(b);
    if (e == cudaSuccess && rc == PBF_OK) e = cudaEventElapsedTime(ms_out, a, b);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "pbf_scene_replay_timed");
    return sync_and_check(s);
}

int pbf_scene_sync(pbf_scene* s) {
    if (!s) return fail(PBF_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    return sync_and_check(s);
}

int pbf_scene_read(pbf_scene* s, int field, float* host_out) {
    if (!s) return fail(PBF_ERR_INVALID_ARG, "scene is NULL");
    if (s->n > 0 && !host_out) return fail(PBF_ERR_INVALID_ARG, "output is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    int rc = PBF_OK;
    switch (field) {
        case PBF_FIELD_POSITIONS: rc = download3(s, s->B.x, host_out, s->n); break;
        case PBF_FIELD_VELOCITIES: rc = download3(s, s->B.v, host_out, s->n); break;
        case PBF_FIELD_DENSITIES:
            if (s->n) PBF_CUDA(cudaMemcpyAsync(host_out, s->B.rho, (size_t)s->n * 4, cudaMemcpyDeviceToHost, s->stream));
            break;
        case PBF_FIELD_LAMBDAS:
            if (s->n) PBF_CUDA(cudaMemcpyAsync(host_out, s->B.lam, (size_t)s->n * 4, cudaMemcpyDeviceToHost, s->stream));
            break;
        default: return fail(PBF_ERR_INVALID_ARG, "unknown field");
    }
    if (rc) return rc;
    return sync_and_check(s);
}

int pbf_scene_write(pbf_scene* s, int field, const float* host_in) {
    if (!s) return fail(PBF_ERR_INVALID_ARG, "scene is NULL");
    if (s->n > 0 && !host_in) return fail(PBF_ERR_INVALID_ARG, "input is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    int rc = PBF_OK;
    switch (field) {
        case PBF_FIELD_POSITIONS:
            rc = upload3(s, host_in, s->B.x, s->n);
            if (!rc) update_bbox(s, host_in, s->n);
            break;
        case PBF_FIELD_VELOCITIES: rc = upload3(s, host_in, s->B.v, s->n); break;
        case PBF_FIELD_DENSITIES:
            if (s->n) PBF_CUDA(cudaMemcpyAsync(s->B.rho, host_in, (size_t)s->n * 4, cudaMemcpyHostToDevice, s->stream));
            break;
        case PBF_FIELD_LAMBDAS:
            if (s->n) PBF_CUDA(cudaMemcpyAsync(s->B.lam, host_in, (size_t)s->n * 4, cudaMemcpyHostToDevice, s->stream));
            break;
        default: return fail(PBF_ERR_INVALID_ARG, "unknown field");
    }
    if (rc) return rc;
    PBF_CUDA(cudaStreamSynchronize(s->stream));
    return PBF_OK;
}

int pbf_scene_device_field(pbf_scene* s, int field, void** dptr) {
    if (!s || !dptr) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    switch (field) {
        case PBF_FIELD_POSITIONS: *dptr = s->B.x; break;
        case PBF_FIELD_VELOCITIES: *dptr = s->B.v; break;
        case PBF_FIELD_DENSITIES: *dptr = s->B.rho; break;
        case PBF_FIELD_LAMBDAS: *dptr = s->B.lam; break;
        default: return fail(PBF_ERR_INVALID_ARG, "unknown field");
    }
    return PBF_OK;
}

int pbf_scene_stream(pbf_scene* s, void** stream) {
    if (!s || !stream) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    *stream = (void*)s->stream;
    return PBF_OK;
}

int pbf_host_alloc(size_t bytes, void** out) {
    if (!out) return fail(PBF_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (bytes == 0) return PBF_OK;
    void* p = nullptr;
    const cudaError_t e = cudaHostAlloc(&p, bytes, cudaHostAllocPortable);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return fail(PBF_ERR_OOM, std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
    }
    *out = p;
    return PBF_OK;
}

int pbf_host_free(void* p) {
    if (!p) return PBF_OK;
    PBF_CUDA(cudaFreeHost(p));
    return PBF_OK;
}

int pbf_solver_step_host(pbf_scene* s, int n, float* x3, float* v3, float* densities,
                         float* lambdas, float dt, const float* g3, float mass) {
    if (!s) return fail(PBF_ERR_INVALID_ARG, "scene is NULL");
    if (n == 0) return PBF_OK;  // pbf_solver.cpp:21
    if (n < 0 || !x3 || !v3 || !densities || !lambdas || !g3)
        return fail(PBF_ERR_INVALID_ARG, "NULL argument or negative n");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    int rc = set_state(s, n, x3, v3);
    if (rc) return rc;
    PBF_CUDA(cudaMemcpyAsync(s->B.rho, densities, (size_t)n * 4, cudaMemcpyHostToDevice, s->stream));
    PBF_CUDA(cudaMemcpyAsync(s->B.lam, lambdas, (size_t)n * 4, cudaMemcpyHostToDevice, s->stream));
    for (int d = 0; d < 3; ++d) s->gravity[d] = g3[d];
    s->mass = mass;
    rc = run_steps(s, dt, 1);
    if (rc) return rc;
    rc = download3(s, s->B.x, x3, n);
    if (rc) return rc;
    rc = download3(s, s->B.v, v3, n);
    if (rc) return rc;
    PBF_CUDA(cudaMemcpyAsync(densities, s->B.rho, (size_t)n * 4, cudaMemcpyDeviceToHost, s->stream));
    PBF_CUDA(cudaMemcpyAsync(lambdas, s->B.lam, (size_t)n * 4, cudaMemcpyDeviceToHost, s->stream));
    return sync_and_check(s);
}

int pbf_scene_check_finite(pbf_scene* s) {
    if (!s) return fail(PBF_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    if (s->n == 0) return PBF_OK;
    if (!s->d_flag) PBF_CUDA(cudaMalloc(&s->d_flag, 4));
    PBF_CUDA(cudaMemsetAsync(s->d_flag, 0, 4, s->stream));
    k_finite<<<(s->n + 255) / 256, 256, 0, s->stream>>>(s->B.x, s->B.v, s->n, s->d_flag);
    PBF_CUDA(cudaGetLastError());
    uint32_t f = 0;
    PBF_CUDA(cudaMemcpyAsync(&f, s->d_flag, 4, cudaMemcpyDeviceToHost, s->stream));
    PBF_CUDA(cudaStreamSynchronize(s->stream));
    if (f) return fail(PBF_ERR_NONFINITE, "non-finite particle position or velocity");
    return PBF_OK;
}

int pbf_scene_debug_cells(pbf_scene* s, float dt, int* cells3) {
    if (!s || (s->n > 0 && !cells3)) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    if (s->n == 0) return PBF_OK;
    StepConsts C;
    int rc = make_consts(s, dt, C);
    if (rc) return rc;
    int* d = nullptr;
    PBF_CUDA(cudaMalloc(&d, (size_t)s->n * 12));
    cudaError_t e = debug_cells(s->B, C, d, s->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(cells3, d, (size_t)s->n * 12, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "debug_cells");
    return PBF_OK;
}

int pbf_scene_debug_neighbors(pbf_scene* s, float dt, long long* offsets, int* out_idx,
                              long long cap, long long* total) {
    if (!s || !offsets || !total) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    const int n = s->n;
    *total = 0;
    offsets[0] = 0;
    if (n == 0) return PBF_OK;
    StepConsts C;
    int rc = make_consts(s, dt, C);
    if (rc) return rc;
    long long* d_cnt = nullptr;
    long long* d_offs = nullptr;
    int* d_out = nullptr;
    std::vector<long long> cnt(n);
    cudaError_t e = cudaMalloc(&d_cnt, (size_t)n * 8);
    if (e == cudaSuccess) e = debug_neighbors(s->B, C, s->sort, d_cnt, nullptr, nullptr, 0, 0, s->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(cnt.data(), d_cnt, (size_t)n * 8, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    long long tot = 0;
    for (int i = 0; i < n; ++i) {
        offsets[i] = tot;
        tot += cnt[i];
    }
    offsets[n] = tot;
    *total = tot;
    if (e == cudaSuccess && out_idx && cap > 0) {
        e = cudaMalloc(&d_offs, (size_t)(n + 1) * 8);
        if (e == cudaSuccess) e = cudaMalloc(&d_out, (size_t)std::max<long long>(cap, 1) * 4);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_offs, offsets, (size_t)(n + 1) * 8, cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess)
            e = debug_neighbors(s->B, C, s->sort, nullptr, d_offs, d_out, cap, 1, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(out_idx, d_out, (size_t)std::min(cap, tot) * 4,
                                cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    }
    if (d_cnt) cudaFree(d_cnt);
    if (d_offs) cudaFree(d_offs);
    if (d_out) cudaFree(d_out);
    if (e != cudaSuccess) return cuda_fail(e, "debug_neighbors");
    // Canonical sets: ascending, duplicates (double-visited buckets) removed.
    if (out_idx && cap >= tot) {
        long long w = 0;
        for (int i = 0; i < n; ++i) {
            const long long a = offsets[i], b = offsets[i + 1];
            std::sort(out_idx + a, out_idx + b);
            const long long start = w;
            for (long long k = a; k < b; ++k)
                if (k == a || out_idx[k] != out_idx[k - 1]) out_idx[w++] = out_idx[k];
            offsets[i] = start;
        }
        offsets[n] = w;
        *total = w;
    }
    return sync_and_check(s);
}

const char* pbf_phase_name(int phase) {
    // Scope names of the reference's PerformanceMonitor (pbf_solver.cpp:29-103).
    static const char* names[kNumPhases] = {
        "fluid.pbf.predict",
        "fluid.pbf.grid_build",
        "fluid.pbf.neighbor_query",
        "fluid.pbf.iteration.compute_density",
        "fluid.pbf.iteration.compute_delta_position",
        "fluid.pbf.xsph_viscosity",
        "fluid.pbf.commit_positions",
    };
    return (phase >= 0 && phase < kNumPhases) ? names[phase] : nullptr;
}

int pbf_scene_step_profiled(pbf_scene* s, float dt, float* phase_ms, int* launches) {
    if (!s || !phase_ms) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    for (int k = 0; k < kNumPhases; ++k) {
        phase_ms[k] = 0.0f;
        if (launches) launches[k] = 0;
    }
    if (s->n == 0) return PBF_OK;
    StepConsts C;
    int rc = make_consts(s, dt, C);
    if (rc) return rc;
    PhaseMarks pm;
    int created = 0;
    cudaError_t e = cudaSuccess;
    for (; created < PhaseMarks::kMax && e == cudaSuccess; ++created)
        e = cudaEventCreate(&pm.ev[created]);
    if (e == cudaSuccess) {
        rc = enqueue(s, C, s->stream, &pm);
        if (rc == PBF_OK) e = cudaStreamSynchronize(s->stream);
        for (int k = 1; k < pm.count && e == cudaSuccess && rc == PBF_OK; ++k) {
            float ms = 0.0f;
            e = cudaEventElapsedTime(&ms, pm.ev[k - 1], pm.ev[k]);
            const int ph = pm.phase[k];
            if (ph >= 0 && ph < kNumPhases) {
                phase_ms[ph] += ms;
                if (launches) launches[ph] += pm.launches[k];
            }
        }
    }
    for (int k = 0; k < created; ++k)
        if (pm.ev[k]) cudaEventDestroy(pm.ev[k]);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "pbf_scene_step_profiled");
    return sync_and_check(s);
}

}  // extern "C"

namespace {

// Carves per-boundary-particle arrays for nb particles.
int alloc_boundary(pbf_scene* s, int nb) {
    ++s->buf_gen;
    auto& b = s->bnd;
    for (void* m : {b.mem, b.sort_mem}) if (m) cudaFree(m);
    b.mem = b.sort_mem = nullptr;
    const int c = nb > 0 ? nb : 1;
    const size_t f4 = align_up((size_t)c * 16, 256), f1 = align_up((size_t)c * 4, 256),
                 f2 = align_up((size_t)c * 8, 256), f27 = align_up((size_t)c * 27 * 4, 256);
    const size_t total = 6 * f4 + 9 * f1 + 2 * f2 + f27;
    PBF_CUDA(cudaMalloc(&b.mem, total));
    char* p = reinterpret_cast<char*>(b.mem);
    auto take = [&](size_t n) { char* r = p; p += n; return r; };
    b.local = reinterpret_cast<float4*>(take(f4));
    b.world = reinterpret_cast<float4*>(take(f4));
    b.Fb = reinterpret_cast<float4*>(take(f4));
    b.idx.spos = reinterpret_cast<float4*>(take(f4));
    b.idx.scell = reinterpret_cast<int4*>(take(f4));
    b.bq.qcell = reinterpret_cast<int4*>(take(f4));
    b.body = reinterpret_cast<int*>(take(f1));
    b.idx.keys = reinterpret_cast<uint32_t*>(take(f1));
    b.idx.skeys = reinterpret_cast<uint32_t*>(take(f1));
    b.idx.sidx = reinterpret_cast<uint32_t*>(take(f1));
    b.idx.ridx = reinterpret_cast<uint32_t*>(take(f1));
    b.idx.pos_of = reinterpret_cast<uint32_t*>(take(f1));
    b.idx.kpos = reinterpret_cast<uint32_t*>(take(f1));
    b.idx.bend = reinterpret_cast<uint32_t*>(take(f1));
    b.bq.qown = reinterpret_cast<int*>(take(f1));
    b.idx.rkeys = reinterpret_cast<unsigned long long*>(take(f2));
    b.idx.rsorted = reinterpret_cast<unsigned long long*>(take(f2));
    b.bq.btab = reinterpret_cast<uint32_t*>(take(f27));
    PBF_CUDA(cudaMemsetAsync(b.mem, 0, total, s->stream));
    const size_t sb = sort_scratch_bytes(c);
    PBF_CUDA(cudaMalloc(&b.sort_mem, sb));
    PBF_CUDA(cudaMemsetAsync(b.sort_mem, 0, sb, s->stream));
    sort_scratch_bind(b.sort, b.sort_mem, c);
    b.nb = nb;
    return PBF_OK;
}

int ensure_boundary_grid(pbf_scene* s, uint32_t nslots) {
    auto& b = s->bnd;
    if (b.idx.off && b.idx_slots >= nslots) return PBF_OK;
    ++s->buf_gen;
    if (b.idx.off) cudaFree(b.idx.off);
    b.idx.off = nullptr;
    const size_t ob = align_up((size_t)(nslots + 1) * 4, 256);
    PBF_CUDA(cudaMalloc(&b.idx.off, ob + align_up(nslots, 256)));
    b.idx.slot_alias = reinterpret_cast<unsigned char*>(b.idx.off) + ob;
    b.idx_slots = nslots;
    return PBF_OK;
}

int ensure_fluid_queries(pbf_scene* s) {
    auto& b = s->bnd;
    if (b.fq_mem && b.fq_cap >= s->n) return PBF_OK;
    ++s->buf_gen;
    if (b.fq_mem) cudaFree(b.fq_mem);
    b.fq_mem = nullptr;
    const int c = s->n > 0 ? s->n : 1;
    PBF_CUDA(cudaMalloc(&b.fq_mem, (size_t)c * 16));
    b.fq_cell = reinterpret_cast<int4*>(b.fq_mem);
    b.fq_cap = c;
    return PBF_OK;
}

}  // namespace

extern "C" {

int pbf_scene_set_boundary(pbf_scene* s, int nb, const float* local3, const int* body,
                           const float* psi) {
    if (!s || nb < 0 || (nb > 0 && (!local3 || !body || !psi)))
        return fail(PBF_ERR_INVALID_ARG, "bad boundary arguments");
    if (nb > (1 << 29)) return fail(PBF_ERR_CAPACITY, "at most 2^29 boundary particles");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    int rc = alloc_boundary(s, nb);
    if (rc) return rc;
    auto& b = s->bnd;
    b.nbodies = 0;
    b.needed_bodies = 0;
    ++s->buf_gen;
    if (b.body_mem) cudaFree(b.body_mem);
    b.body_mem = nullptr;
    if (nb == 0) return PBF_OK;
    std::vector<float4> l(nb);
    for (int i = 0; i < nb; ++i)
        l[i] = make_float4(local3[3 * i], local3[3 * i + 1], local3[3 * i + 2], psi[i]);
    PBF_CUDA(cudaMemcpyAsync(b.local, l.data(), (size_t)nb * 16, cudaMemcpyHostToDevice, s->stream));
    PBF_CUDA(cudaMemcpyAsync(b.body, body, (size_t)nb * 4, cudaMemcpyHostToDevice, s->stream));
    // Per-body lists of boundary indices in ascending order (CSR): the
    // reference applies forces to a body in boundary order (fluid_world.cpp:138-172).
    int maxb = -1;
    for (int i = 0; i < nb; ++i) maxb = std::max(maxb, body[i]);
    const int nbody = maxb + 1;
    std::vector<int> off(nbody + 1, 0), lst;
    for (int i = 0; i < nb; ++i)
        if (body[i] >= 0) ++off[body[i] + 1];
    for (int k = 0; k < nbody; ++k) off[k + 1] += off[k];
    lst.resize(off[nbody]);
    std::vector<int> fill(off.begin(), off.end() - 1);
    for (int i = 0; i < nb; ++i)
        if (body[i] >= 0) lst[fill[body[i]]++] = i;
    const int cap = std::max(nbody, 1);
    const size_t s16 = align_up((size_t)cap * 16, 256), s4 = align_up((size_t)(cap + 1) * 4, 256),
                 sl = align_up(std::max<size_t>(lst.size(), 1) * 4, 256),
                 s12 = align_up((size_t)cap * 12, 256);
    const size_t need = 4 * s16 + 2 * s4 + sl + 2 * s12;
    PBF_CUDA(cudaMalloc(&b.body_mem, need));
    char* p = reinterpret_cast<char*>(b.body_mem);
    auto take = [&](size_t n) { char* r = p; p += n; return r; };
    b.body_pos = reinterpret_cast<float4*>(take(s16));
    b.body_quat = reinterpret_cast<float4*>(take(s16));
    b.body_lin = reinterpret_cast<float4*>(take(s16));
    b.body_ang = reinterpret_cast<float4*>(take(s16));
    b.body_dyn = reinterpret_cast<int*>(take(s4));
    b.list_off = reinterpret_cast<int*>(take(s4));
    b.list = reinterpret_cast<int*>(take(sl));
    b.force3 = reinterpret_cast<float*>(take(s12));
    b.torque3 = reinterpret_cast<float*>(take(s12));
    PBF_CUDA(cudaMemsetAsync(b.body_mem, 0, need, s->stream));
    PBF_CUDA(cudaMemcpyAsync(b.list_off, off.data(), off.size() * 4, cudaMemcpyHostToDevice, s->stream));
    if (!lst.empty())
        PBF_CUDA(cudaMemcpyAsync(b.list, lst.data(), lst.size() * 4, cudaMemcpyHostToDevice, s->stream));
    PBF_CUDA(cudaStreamSynchronize(s->stream));
    b.needed_bodies = nbody;
    return PBF_OK;
}

int pbf_scene_set_bodies(pbf_scene* s, int nbodies, const float* pos3, const float* quat4,
                         const int* dynamic) {
    if (!s || nbodies < 0 || (nbodies > 0 && (!pos3 || !quat4 || !dynamic)))
        return fail(PBF_ERR_INVALID_ARG, "bad body arguments");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    auto& b = s->bnd;
    if (!b.body_mem) return fail(PBF_ERR_INVALID_ARG, "set the boundary particles first");
    if (nbodies < b.needed_bodies)
        return fail(PBF_ERR_INVALID_ARG, "fewer bodies than the boundary particles reference");
    // Bodies past the last one with boundary particles receive no coupling.
    nbodies = b.needed_bodies;
    std::vector<float4> bp(nbodies), bq(nbodies);
    for (int k = 0; k < nbodies; ++k) {
        bp[k] = make_float4(pos3[3 * k], pos3[3 * k + 1], pos3[3 * k + 2], 0.0f);
        bq[k] = make_float4(quat4[4 * k], quat4[4 * k + 1], quat4[4 * k + 2], quat4[4 * k + 3]);
    }
    if (nbodies > 0) {
        PBF_CUDA(cudaMemcpyAsync(b.body_pos, bp.data(), (size_t)nbodies * 16, cudaMemcpyHostToDevice, s->stream));
        PBF_CUDA(cudaMemcpyAsync(b.body_quat, bq.data(), (size_t)nbodies * 16, cudaMemcpyHostToDevice, s->stream));
        PBF_CUDA(cudaMemcpyAsync(b.body_dyn, dynamic, (size_t)nbodies * 4, cudaMemcpyHostToDevice, s->stream));
    }
    PBF_CUDA(cudaStreamSynchronize(s->stream));
    b.nbodies = nbodies;
    return PBF_OK;
}

int pbf_scene_set_body_velocities(pbf_scene* s, int nbodies, const float* lin3,
                                  const float* ang3) {
    if (!s || nbodies < 0 || (nbodies > 0 && (!lin3 || !ang3)))
        return fail(PBF_ERR_INVALID_ARG, "bad body velocity arguments");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    auto& b = s->bnd;
    if (!b.body_mem) return fail(PBF_ERR_INVALID_ARG, "set the boundary particles first");
    if (nbodies < b.needed_bodies)
        return fail(PBF_ERR_INVALID_ARG, "fewer bodies than the boundary particles reference");
    nbodies = b.needed_bodies;
    std::vector<float4> lv(nbodies), av(nbodies);
    for (int k = 0; k < nbodies; ++k) {
        lv[k] = make_float4(lin3[3 * k], lin3[3 * k + 1], lin3[3 * k + 2], 0.0f);
        av[k] = make_float4(ang3[3 * k], ang3[3 * k + 1], ang3[3 * k + 2], 0.0f);
    }
    if (nbodies > 0) {
        PBF_CUDA(cudaMemcpyAsync(b.body_lin, lv.data(), (size_t)nbodies * 16, cudaMemcpyHostToDevice, s->stream));
        PBF_CUDA(cudaMemcpyAsync(b.body_ang, av.data(), (size_t)nbodies * 16, cudaMemcpyHostToDevice, s->stream));
    }
    PBF_CUDA(cudaStreamSynchronize(s->stream));
    return PBF_OK;
}

}  // extern "C"

namespace {

// Enqueues on the scene's stream: boundary world positions from the current
// body poses, boundary density added to the final densities, coupling forces
// and torques accumulated onto the device accumulators b.force3 / b.torque3,
// which start from force_in / torque_in (host arrays) or from zero
// (fluid_world.cpp:57-81 after the PBF step).  C are the constants of the step
// that produced the current state.  Needs b.nb > 0.
int enqueue_coupling(pbf_scene* s, const StepConsts& C, const float* force_in,
                     const float* torque_in, cudaEvent_t* marks = nullptr,
                     bool density_has_boundary = false) {
    auto& b = s->bnd;
    const int nbodies = b.nbodies;
    cudaStream_t st = s->stream;
    // marks[0..3]: start, after the positions, after the density, end
    auto mark = [&](int k) { return marks ? cudaEventRecord(marks[k], st) : cudaSuccess; };
    PBF_CUDA(mark(0));
    // 1. boundary world positions from the step-start transforms (unchanged
    //    by the PBF step, which never reads the boundary)
    cudaError_t e = boundary_xform(b.local, b.body, b.nb, b.body_pos, b.body_quat, nbodies,
                                   b.world, st);
    if (e == cudaSuccess) e = mark(1);
    if (e != cudaSuccess) return cuda_fail(e, "boundary_xform");
    // 2. boundary density on the final positions (fluid_world.cpp:101-123)
    int rc = ensure_boundary_grid(s, C.grid.nslots);
    if (rc) return rc;
    rc = ensure_fluid_queries(s);
    if (rc) return rc;
    e = index_build(b.idx, b.world, nullptr, b.nb, C, b.sort, st);
    QuerySet fq{b.fq_cell, s->B.sown, s->B.btab};
    // A two-way step's densities already hold the boundary's share (from
    // its last Jacobi iteration).
    if (!density_has_boundary) {
        if (e == cudaSuccess) e = index_classify(fq, s->B.x, s->n, b.idx, C, st);
        if (e == cudaSuccess) e = boundary_density(s->B.x, s->n, fq, b.idx, s->B.rho, C, st);
    }
    if (e == cudaSuccess) e = mark(2);
    if (e != cudaSuccess) return cuda_fail(e, "boundary density");
    // 3. coupling forces from a fresh fluid grid on the final positions
    //    (fluid_world.cpp:125-174); the step's sorted buffers are free now.
    PointIndex fidx;
    fidx.keys = s->B.keys;
    fidx.skeys = s->B.skeys;
    fidx.sidx = s->B.sidx;
    fidx.rkeys = s->B.rkeys;
    fidx.rsorted = s->B.rsorted;
    fidx.ridx = s->B.ridx;
    fidx.pos_of = s->B.pos_of;
    fidx.kpos = s->B.kpos;
    fidx.bend = s->B.bend;
    fidx.spos = s->B.xb;
    fidx.scell = s->B.scell;
    fidx.off = s->B.off;
    fidx.slot_alias = s->B.slot_alias;
    e = index_build(fidx, s->B.x, s->B.rho, s->n, C, s->sort, st);
    if (e == cudaSuccess) e = index_classify(b.bq, b.world, b.nb, fidx, C, st);
    if (e == cudaSuccess)
        e = coupling_forces(b.world, b.body, b.body_dyn, b.nb, nbodies, b.bq, fidx, b.Fb, C, st);
    if (nbodies > 0) {
        const size_t bytes = (size_t)nbodies * 12;
        if (e == cudaSuccess)
            e = force_in ? cudaMemcpyAsync(b.force3, force_in, bytes, cudaMemcpyHostToDevice, st)
                         : cudaMemsetAsync(b.force3, 0, bytes, st);
        if (e == cudaSuccess)
            e = torque_in ? cudaMemcpyAsync(b.torque3, torque_in, bytes, cudaMemcpyHostToDevice, st)
                          : cudaMemsetAsync(b.torque3, 0, bytes, st);
        if (e == cudaSuccess)
            // The exact build keeps the reference's serial order; the fast
            // build reduces each body's terms as a tree.
            e = body_reduce(b.Fb, b.world, b.list_off, b.list, b.body_pos, nbodies, b.force3,
                            b.torque3, !s->settings.exact_arithmetic, st);
    }
    if (e == cudaSuccess) e = mark(3);
    if (e != cudaSuccess) return cuda_fail(e, "coupling forces");
    return PBF_OK;
}

// The coupling after a step, with the forces and torques added onto the host
// arrays force3 / torque3; waits for it.
// With phase_ms (3 entries), also the device time of the boundary positions,
// the boundary density and the coupling forces.
int couple_after_step(pbf_scene* s, const StepConsts& C, float* force3, float* torque3,
                      float* phase_ms = nullptr, bool density_has_boundary = false) {
    auto& b = s->bnd;
    if (phase_ms)
        for (int k = 0; k < 3; ++k) phase_ms[k] = 0.0f;
    if (b.nb == 0) return sync_and_check(s);
    cudaEvent_t ev[4] = {};
    int created = 0;
    if (phase_ms)
        for (; created < 4; ++created)
            if (cudaEventCreate(&ev[created]) != cudaSuccess) break;
    auto destroy = [&] {
        for (int k = 0; k < created; ++k) cudaEventDestroy(ev[k]);
    };
    if (phase_ms && created < 4) {
        destroy();
        return cuda_fail(cudaGetLastError(), "cudaEventCreate");
    }
    int rc = enqueue_coupling(s, C, force3, torque3, phase_ms ? ev : nullptr,
                              density_has_boundary);
    if (!rc && b.nbodies > 0) {
        const size_t bytes = (size_t)b.nbodies * 12;
        cudaError_t e = cudaMemcpyAsync(force3, b.force3, bytes, cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(torque3, b.torque3, bytes, cudaMemcpyDeviceToHost, s->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "coupling forces copy");
    }
    if (!rc) rc = sync_and_check(s);
    if (!rc && phase_ms)
        for (int k = 0; k < 3; ++k)
            if (cudaEventElapsedTime(&phase_ms[k], ev[k], ev[k + 1]) != cudaSuccess) {
                rc = cuda_fail(cudaGetLastError(), "cudaEventElapsedTime");
                break;
            }
    destroy();
    return rc;
}

}  // namespace

namespace pbf {
namespace capi {

int scene_set_rigid(pbf_scene* s, int nbodies, const pbf_rigid_body* bodies) {
    if (!s || nbodies < 0 || (nbodies > 0 && !bodies))
        return fail(PBF_ERR_INVALID_ARG, "bad body arguments");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    auto& b = s->bnd;
    ++s->buf_gen;
    if (b.rb) cudaFree(b.rb);
    b.rb = nullptr;
    b.nrb = 0;
    if (nbodies == 0) return PBF_OK;
    PBF_CUDA(cudaMalloc(&b.rb, (size_t)nbodies * sizeof(pbf_rigid_body)));
    PBF_CUDA(cudaMemcpyAsync(b.rb, bodies, (size_t)nbodies * sizeof(pbf_rigid_body),
                             cudaMemcpyHostToDevice, s->stream));
    PBF_CUDA(cudaStreamSynchronize(s->stream));
    b.nrb = nbodies;
    return PBF_OK;
}

int scene_set_contacts(pbf_scene* s, int nshapes, const pbf_rigid_shape* shapes,
                       const pbf_contact_settings* cs) {
    if (!s || nshapes < 0 || (nshapes > 0 && !shapes))
        return fail(PBF_ERR_INVALID_ARG, "bad shape arguments");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    auto& b = s->bnd;
    if (nshapes > 16 || b.nrb > 16)
        return fail(PBF_ERR_INVALID_ARG, "rigid contacts take at most 16 shapes and 16 bodies");
    for (int k = 0; k < nshapes; ++k) {
        const pbf_rigid_shape& sh = shapes[k];
        if (sh.type == PBF_SHAPE_SPHERE) {
            if (sh.body >= b.nrb || sh.body < -1)
                return fail(PBF_ERR_INVALID_ARG, "a contact shape names a missing body");
        } else if (sh.type == PBF_SHAPE_PLANE) {
            if (sh.body != -1) return fail(PBF_ERR_INVALID_ARG, "a plane belongs to the world");
        } else {
            return fail(PBF_ERR_INVALID_ARG, "contact shapes are spheres and planes");
        }
    }
    if (cs && cs->velocity_iterations < 0)
        return fail(PBF_ERR_INVALID_ARG, "velocity_iterations must be >= 0");
    ++s->buf_gen;
    if (b.shapes) cudaFree(b.shapes);
    b.shapes = nullptr;
    b.nshapes = 0;
    if (cs) b.cset = *cs;
    if (nshapes == 0) return PBF_OK;
    PBF_CUDA(cudaMalloc(&b.shapes, (size_t)nshapes * sizeof(pbf_rigid_shape)));
    PBF_CUDA(cudaMemcpyAsync(b.shapes, shapes, (size_t)nshapes * sizeof(pbf_rigid_shape),
                             cudaMemcpyHostToDevice, s->stream));
    PBF_CUDA(cudaStreamSynchronize(s->stream));
    b.nshapes = nshapes;
    return PBF_OK;
}

int scene_read_rigid(pbf_scene* s, pbf_rigid_body* out) {
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    auto& b = s->bnd;
    if (b.nrb > 0)
        PBF_CUDA(cudaMemcpyAsync(out, b.rb, (size_t)b.nrb * sizeof(pbf_rigid_body),
                                 cudaMemcpyDeviceToHost, s->stream));
    return sync_and_check(s);
}

int scene_couple_rigid_async(pbf_scene* s, float dt, const float g[3]) {
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    return scene_couple_rigid_locked(s, dt, g);
}

int scene_couple_rigid_locked(pbf_scene* s, float dt, const float g[3]) {
    auto& b = s->bnd;
    if (b.nb > 0 && b.nbodies < b.needed_bodies) return fail(PBF_ERR_INVALID_ARG, "set the bodies first");
    const bool couple = s->n > 0 && b.nb > 0;  // fluid_world.cpp:57
    pbf_scene::CoupleKey key;
    key.valid = true;
    if (couple) {
        // Every allocation happens here, before any capture.
        int rc = make_consts(s, dt, key.C);
        if (!rc) rc = ensure_boundary_grid(s, key.C.grid.nslots);
        if (!rc) rc = ensure_fluid_queries(s);
        if (rc) return rc;
    }
    key.dt = dt;
    for (int d = 0; d < 3; ++d) key.g[d] = g[d];
    key.n = s->n;
    key.nb = b.nb;
    key.nbodies = b.nbodies;
    key.nrb = b.nrb;
    key.gen = s->buf_gen;
    auto same = [](const pbf_scene::CoupleKey& x, const pbf_scene::CoupleKey& y) {
        return x.valid && y.valid && consts_equal(x.C, y.C) && x.dt == y.dt && x.g[0] == y.g[0] &&
               x.g[1] == y.g[1] && x.g[2] == y.g[2] && x.n == y.n && x.nb == y.nb &&
               x.nbodies == y.nbodies && x.nrb == y.nrb && x.gen == y.gen;
    };
    auto enqueue_all = [&]() -> int {
        if (couple) {
            const int rc = enqueue_coupling(s, key.C, nullptr, nullptr);
            if (rc) return rc;
        }
        const int nforce = couple ? b.nbodies : 0;
        if (b.nshapes > 0) {
            const cudaError_t e = rigid_world(b.rb, b.nrb, b.shapes, b.nshapes, b.cset, b.force3,
                                              b.torque3, nforce, g[0], g[1], g[2], dt, b.body_pos,
                                              b.body_quat, s->stream);
            return e == cudaSuccess ? PBF_OK : cuda_fail(e, "rigid contacts");
        }
        const cudaError_t e = rigid_step(b.rb, b.nrb, b.force3, b.torque3, nforce, g[0], g[1], g[2],
                                         dt, b.body_pos, b.body_quat, s->stream);
        return e == cudaSuccess ? PBF_OK : cuda_fail(e, "rigid step");
    };
    if (!graphs_enabled()) return enqueue_all();
    if (!(s->couple_graph && same(key, s->couple_key))) {
        if (!same(key, s->couple_seen)) {
            // A key seen once runs directly; the second time in a row it is captured.
            s->couple_seen = key;
            return enqueue_all();
        }
        if (s->couple_graph) {
            cudaGraphExecDestroy(s->couple_graph);
            s->couple_graph = nullptr;
        }
        cudaGraph_t gr = nullptr;
        PBF_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        const int erc = enqueue_all();
        cudaError_t ce = cudaStreamEndCapture(s->stream, &gr);
        if (erc) {
            if (gr) cudaGraphDestroy(gr);
            return erc;
        }
        if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
        ce = cudaGraphInstantiate(&s->couple_graph, gr, 0);
        cudaGraphDestroy(gr);
        if (ce != cudaSuccess) {
            s->couple_graph = nullptr;
            return cuda_fail(ce, "cudaGraphInstantiate");
        }
        s->couple_key = key;
    }
    PBF_CUDA(cudaGraphLaunch(s->couple_graph, s->stream));
    return PBF_OK;
}

}  // namespace capi
}  // namespace pbf

namespace {

// Buffers of a two-way step: predicted positions, their cells, owner words
// and bucket rows, per fluid particle.
int ensure_two_way(pbf_scene* s) {
    auto& b = s->bnd;
    if (b.tw_mem && b.tw_cap >= s->n) return PBF_OK;
    if (b.tw_mem) cudaFree(b.tw_mem);
    b.tw_mem = nullptr;
    const size_t c = (size_t)(s->n > 0 ? s->n : 1);
    const size_t pb = align_up(c * 16, 256), cb = align_up(c * 16, 256), ob = align_up(c * 4, 256);
    PBF_CUDA(cudaMalloc(&b.tw_mem, pb + cb + ob + c * 27 * 4));
    unsigned char* m = static_cast<unsigned char*>(b.tw_mem);
    b.tw_pred = reinterpret_cast<float4*>(m);
    b.tw_cell = reinterpret_cast<int4*>(m + pb);
    b.tw_own = reinterpret_cast<int*>(m + pb + cb);
    b.tw_btab = reinterpret_cast<uint32_t*>(m + pb + cb + ob);
    b.tw_cap = (int)c;
    return PBF_OK;
}

// One PBF step with the Akinci boundary inside the density constraint
// (pbf_settings.boundary_two_way): the boundary's world positions at the
// step-start poses, the reference-bucket index over them, every fluid
// particle's predicted cell classified against it, then the step.
int two_way_step(pbf_scene* s, const StepConsts& C) {
    auto& b = s->bnd;
    int rc = ensure_boundary_grid(s, C.grid.nslots);
    if (!rc) rc = ensure_two_way(s);
    if (rc) return rc;
    cudaStream_t st = s->stream;
    cudaError_t e = boundary_xform(b.local, b.body, b.nb, b.body_pos, b.body_quat, b.nbodies,
                                   b.world, st);
    if (e == cudaSuccess) e = index_build(b.idx, b.world, nullptr, b.nb, C, b.sort, st);
    if (e == cudaSuccess) e = predict_points(s->B.x, s->B.v, s->n, b.tw_pred, C, st);
    QuerySet q{b.tw_cell, b.tw_own, b.tw_btab};
    if (e == cudaSuccess) e = index_classify(q, b.tw_pred, s->n, b.idx, C, st);
    if (e != cudaSuccess) return cuda_fail(e, "two-way boundary");
    BoundaryGrid bg;
    bg.spos = b.idx.spos;
    bg.off = b.idx.off;
    bg.kpos = b.idx.kpos;
    bg.bend = b.idx.bend;
    bg.own = b.tw_own;
    bg.btab = b.tw_btab;
    bg.sidx = b.idx.sidx;
    bg.body = b.body;
    bg.nbodies = b.nbodies;
    bg.body_pos = b.body_pos;
    bg.body_lin = b.body_lin;
    bg.body_ang = b.body_ang;
    const int iters = s->settings.solver_iterations;
    e = s->settings.exact_arithmetic
            ? exact_enqueue_step(s->B, C, iters, s->sort, st, nullptr, &bg)
            : fast_enqueue_step(s->B, C, iters, s->sort, st, nullptr, &bg);
    return e == cudaSuccess ? PBF_OK : cuda_fail(e, "two-way step");
}

int check_coupling_args(pbf_scene* s, float* force3, float* torque3) {
    auto& b = s->bnd;
    if (b.nb > 0 && b.nbodies < b.needed_bodies)
        return fail(PBF_ERR_INVALID_ARG, "set the bodies first");
    if (b.nbodies > 0 && (!force3 || !torque3))
        return fail(PBF_ERR_INVALID_ARG, "NULL force/torque");
    return PBF_OK;
}

}  // namespace

extern "C" {

int pbf_scene_step_coupled(pbf_scene* s, float dt, float* force3, float* torque3) {
    if (!s) return fail(PBF_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    int rc = check_coupling_args(s, force3, torque3);
    if (rc) return rc;
    if (s->n == 0) return PBF_OK;  // fluid_world.cpp:57
    StepConsts C;
    rc = make_consts(s, dt, C);
    if (rc) return rc;
    if (C.two_way && s->bnd.nb > 0) {
        rc = two_way_step(s, C);
        if (rc) return rc;
        return couple_after_step(s, C, force3, torque3, nullptr, true);
    }
    rc = run_steps(s, dt, 1);
    if (rc) return rc;
    return couple_after_step(s, C, force3, torque3);
}

int pbf_scene_couple(pbf_scene* s, float dt, float* force3, float* torque3) {
    return pbf_scene_couple_profiled(s, dt, force3, torque3, nullptr);
}

int pbf_scene_couple_profiled(pbf_scene* s, float dt, float* force3, float* torque3,
                              float* phase_ms) {
    if (!s) return fail(PBF_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    if (phase_ms)
        for (int k = 0; k < 3; ++k) phase_ms[k] = 0.0f;
    int rc = check_coupling_args(s, force3, torque3);
    if (rc) return rc;
    if (s->n == 0) return PBF_OK;
    StepConsts C;
    rc = make_consts(s, dt, C);
    if (rc) return rc;
    return couple_after_step(s, C, force3, torque3, phase_ms);
}

int pbf_scene_read_boundary(pbf_scene* s, float* world3) {
    if (!s || (s->bnd.nb > 0 && !world3)) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    DeviceGuard dg(s->device);
    auto& b = s->bnd;
    if (b.nb == 0) return PBF_OK;
    std::vector<float4> w(b.nb);
    PBF_CUDA(cudaMemcpyAsync(w.data(), b.world, (size_t)b.nb * 16, cudaMemcpyDeviceToHost, s->stream));
    PBF_CUDA(cudaStreamSynchronize(s->stream));
    for (int i = 0; i < b.nb; ++i) {
        world3[3 * i] = w[i].x;
        world3[3 * i + 1] = w[i].y;
        world3[3 * i + 2] = w[i].z;
    }
    return PBF_OK;
}

int pbf_boundary_volumes(int device, int nb, const float* world3, float kernel_radius,
                         float* psi_out) {
    if (nb < 0 || (nb > 0 && (!world3 || !psi_out)))
        return fail(PBF_ERR_INVALID_ARG, "bad arguments");
    if (!(kernel_radius > 0.0f)) return fail(PBF_ERR_INVALID_ARG, "kernel_radius must be > 0");
    if (nb == 0) return PBF_OK;
    // A scratch scene whose "fluid" is the boundary sample: reuses the grid fit.
    pbf_settings st;
    pbf_default_settings(&st);
    st.kernel_radius = kernel_radius;
    pbf_scene* s = nullptr;
    int rc = pbf_scene_create(device, &st, 0, nullptr, nullptr, 0.0f, &s);
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        DeviceGuard dg(s->device);
        update_bbox(s, world3, nb);
        StepConsts C;
        rc = make_consts(s, 1.0f, C);
        std::vector<int> bodies(nb, -1);
        std::vector<float> zero(nb, 0.0f);
        if (!rc) rc = alloc_boundary(s, nb);
        if (!rc) rc = ensure_boundary_grid(s, C.grid.nslots);
        auto& b = s->bnd;
        cudaError_t e = cudaSuccess;
        if (!rc) {
            std::vector<float4> l(nb);
            for (int i = 0; i < nb; ++i)
                l[i] = make_float4(world3[3 * i], world3[3 * i + 1], world3[3 * i + 2], 0.0f);
            e = cudaMemcpyAsync(b.world, l.data(), (size_t)nb * 16, cudaMemcpyHostToDevice, s->stream);
            if (e == cudaSuccess) e = index_build(b.idx, b.world, nullptr, nb, C, b.sort, s->stream);
            if (e == cudaSuccess) e = index_classify(b.bq, b.world, nb, b.idx, C, s->stream);
            float* dpsi = reinterpret_cast<float*>(b.Fb);
            if (e == cudaSuccess) e = boundary_volumes(b.world, nb, b.bq, b.idx, dpsi, C, s->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(psi_out, dpsi, (size_t)nb * 4, cudaMemcpyDeviceToHost, s->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
            if (e != cudaSuccess) rc = cuda_fail(e, "pbf_boundary_volumes");
        }
    }
    const int rc2 = pbf_scene_destroy(s);
    return rc ? rc : rc2;
}

int pbf_sort_pairs_host(int device, int n, const unsigned* keys, int key_bits, unsigned* out_keys,
                        unsigned* out_vals) {
    if (n < 0 || (n > 0 && (!keys || !out_keys || !out_vals)))
        return fail(PBF_ERR_INVALID_ARG, "bad arguments");
    if (key_bits < 1 || key_bits > 32) return fail(PBF_ERR_INVALID_ARG, "key_bits in [1, 32]");
    if (n == 0) return PBF_OK;
    DeviceGuard dg(device);
    if (!dg.ok) return fail(PBF_ERR_NO_DEVICE, "cudaSetDevice failed");
    uint32_t *dk = nullptr, *dko = nullptr, *dvo = nullptr;
    void* scratch = nullptr;
    SortScratch ss;
    cudaError_t e = cudaMalloc(&dk, (size_t)n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dko, (size_t)n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dvo, (size_t)n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&scratch, sort_scratch_bytes(n));
    if (e == cudaSuccess) e = cudaMemset(scratch, 0, sort_scratch_bytes(n));
    if (e == cudaSuccess) {
        sort_scratch_bind(ss, scratch, n);
        e = cudaMemcpy(dk, keys, (size_t)n * 4, cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = radix_sort_pairs(dk, dko, dvo, n, key_bits, ss, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    uint32_t err = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&err, ss.err, 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(out_keys, dko, (size_t)n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(out_vals, dvo, (size_t)n * 4, cudaMemcpyDeviceToHost);
    cudaFree(dk);
    cudaFree(dko);
    cudaFree(dvo);
    cudaFree(scratch);
    if (e != cudaSuccess) return cuda_fail(e, "pbf_sort_pairs_host");
    if (err) return fail(PBF_ERR_TIMEOUT, "device-side wait in the sort gave up");
    return PBF_OK;
}

}  // extern "C"
