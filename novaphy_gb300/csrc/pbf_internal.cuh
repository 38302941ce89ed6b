// Internals shared by the translation units of the C ABI (pbf_capi.cu,
// pbf_batch.cu): error reporting, the device guard and the scene object.
#pragma once

#include <cstddef>
#include <mutex>
#include <string>

#include "novaphy_pbf.h"
#include "pbf_boundary.cuh"
#include "pbf_types.cuh"
#include "radix_sort.cuh"

namespace pbf {
namespace capi {

// Records `msg` as the calling thread's pbf_last_error() and returns `code`.
int fail(int code, const std::string& msg);
// Maps a CUDA error to a PBF status (allocation failure -> PBF_ERR_OOM).
int cuda_fail(cudaError_t e, const char* where);

#define PBF_CUDA(expr)                                           \
    do {                                                         \
        cudaError_t e_ = (expr);                                 \
        if (e_ != cudaSuccess) return ::pbf::capi::cuda_fail(e_, #expr); \
    } while (0)

// Sets the device for the lifetime of the guard, restoring the previous one.
struct DeviceGuard {
    int prev = -1;
    bool ok = false;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        ok = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Device bytes per particle of a scene's resident state: x, v (float4),
// rho, lambda (float) and the float3 staging buffer.
constexpr size_t kStateBytesPerParticle = 16 + 16 + 4 + 4 + 12;

// Step scratch of c particles, carved from one allocation: the sorted
// copies (sx, xa, xb, sv, sv2, som, scell: float4/int4), srho, the cell keys
// and permutation, the reference keys, buckets and classification rows.
inline size_t work_bytes(int c) {
    const size_t f4 = align_up((size_t)c * 16, 256);
    const size_t f1 = align_up((size_t)c * 4, 256);
    const size_t f2 = align_up((size_t)c * 8, 256);
    const size_t f27 = align_up((size_t)c * 27 * 4, 256);
    return 7 * f4 + 9 * f1 + 2 * f2 + f27;
}

inline void bind_work(StepBuffers& B, void* mem, int c) {
    const size_t f4 = align_up((size_t)c * 16, 256);
    const size_t f1 = align_up((size_t)c * 4, 256);
    const size_t f2 = align_up((size_t)c * 8, 256);
    char* p = reinterpret_cast<char*>(mem);
    auto take = [&](size_t b) {
        char* r = p;
        p += b;
        return r;
    };
    B.sx = reinterpret_cast<float4*>(take(f4));
    B.xa = reinterpret_cast<float4*>(take(f4));
    B.xb = reinterpret_cast<float4*>(take(f4));
    B.sv = reinterpret_cast<float4*>(take(f4));
    B.sv2 = reinterpret_cast<float4*>(take(f4));
    B.som = reinterpret_cast<float4*>(take(f4));
    B.scell = reinterpret_cast<int4*>(take(f4));
    B.srho = reinterpret_cast<float*>(take(f1));
    B.keys = reinterpret_cast<uint32_t*>(take(f1));
    B.skeys = reinterpret_cast<uint32_t*>(take(f1));
    B.sidx = reinterpret_cast<uint32_t*>(take(f1));
    B.ridx = reinterpret_cast<uint32_t*>(take(f1));
    B.pos_of = reinterpret_cast<uint32_t*>(take(f1));
    B.kpos = reinterpret_cast<uint32_t*>(take(f1));
    B.bend = reinterpret_cast<uint32_t*>(take(f1));
    B.sown = reinterpret_cast<int*>(take(f1));
    B.rkeys = reinterpret_cast<unsigned long long*>(take(f2));
    B.rsorted = reinterpret_cast<unsigned long long*>(take(f2));
    B.btab = reinterpret_cast<uint32_t*>(p);
}

}  // namespace capi
}  // namespace pbf

struct pbf_scene {
    int device = 0;
    cudaStream_t stream = nullptr;      // where the scene's work is ordered
    cudaStream_t own_stream = nullptr;  // the stream created with the scene
    std::mutex mu;
    pbf_settings settings{};
    float gravity[3] = {0.0f, -9.81f, 0.0f};  // World default (include/novaphy/sim/world.h:157)
    float mass = 0.0f;
    int n = 0;
    int cap = 0;       // particles the state arrays hold
    int work_cap = 0;  // particles the step scratch holds (allocated on first step)
    // Region the grid is fitted to when the domain clamp is off.
    bool have_bbox = false;
    float bbox_lo[3] = {0, 0, 0}, bbox_hi[3] = {0, 0, 0};

    void* pmem = nullptr;  // resident state: x, v, rho, lambda, staging
    void* wmem = nullptr;  // step scratch (sorted copies, keys, buckets)
    void* smem = nullptr;  // sort scratch
    uint32_t* off = nullptr;
    uint32_t off_cap = 0;  // entries
    float* staging = nullptr;  // float[3 cap]
    uint32_t* d_flag = nullptr;
    cudaEvent_t ev = nullptr;  // orders a batch after the scene's own stream
    pbf::SortScratch sort{};
    pbf::StepBuffers B{};

    // Graph of one step, re-captured when the constants change.
    cudaGraphExec_t graph = nullptr;
    pbf::StepConsts graph_consts{};
    int graph_iters = -1;
    int graph_exact = -1;

    // Bumped whenever a device buffer that a captured graph uses is
    // reallocated, so such graphs are captured anew.
    unsigned long long buf_gen = 0;
    // Graph of the post-step of a served coupled scene (coupling and rigid
    // step, scene_couple_rigid_async), captured the second time in a row the
    // same key is seen.
    struct CoupleKey {
        bool valid = false;
        pbf::StepConsts C{};
        float dt = 0.0f, g[3] = {0.0f, 0.0f, 0.0f};
        int n = 0, nb = 0, nbodies = 0, nrb = 0;
        unsigned long long gen = 0;
    };
    cudaGraphExec_t couple_graph = nullptr;
    CoupleKey couple_key, couple_seen;

    // Akinci boundary (FluidWorld coupling).
    struct Boundary {
        int nb = 0, nbodies = 0, needed_bodies = 0;
        void* mem = nullptr;       // per-boundary-particle arrays
        void* body_mem = nullptr;  // per-body arrays
        void* sort_mem = nullptr;
        void* fq_mem = nullptr;    // fluid-query cells (per fluid particle)
        int fq_cap = 0;
        // Two-way coupled steps: predicted fluid positions and their
        // classification against the boundary index (per fluid particle).
        void* tw_mem = nullptr;
        int tw_cap = 0;
        float4* tw_pred = nullptr;
        int4* tw_cell = nullptr;
        int* tw_own = nullptr;
        uint32_t* tw_btab = nullptr;
        float4* local = nullptr;   // w = psi
        int* body = nullptr;
        float4* world = nullptr;   // w = psi
        float4* Fb = nullptr;
        pbf::PointIndex idx;       // reference buckets over the boundary
        pbf::QuerySet bq;          // boundary queries against the fluid index
        int4* fq_cell = nullptr;
        float4* body_pos = nullptr;
        float4* body_quat = nullptr;
        float4* body_lin = nullptr;  // body velocities (two-way boundary friction)
        float4* body_ang = nullptr;
        int* body_dyn = nullptr;
        int* list_off = nullptr;
        int* list = nullptr;
        float* force3 = nullptr;
        float* torque3 = nullptr;
        pbf::SortScratch sort{};
        uint32_t idx_slots = 0;
        // Device copy of all rigid bodies when they step on the device
        // (served coupled scenes), else null.
        pbf_rigid_body* rb = nullptr;
        int nrb = 0;
        // Contact shapes of those bodies (device copy), when they collide.
        pbf_rigid_shape* shapes = nullptr;
        int nshapes = 0;
        pbf_contact_settings cset{30, 0.3f, 0.005f, 1};
    } bnd;
};

struct pbf_snapshot {
    int device = 0;
    int n = 0;
    pbf_settings settings{};
    float gravity[3] = {0, 0, 0};
    float mass = 0.0f;
    void* mem = nullptr;  // x (float4 n) | v (float4 n) | rho (n) | lam (n)
};

namespace pbf {
namespace capi {

int check_settings(const pbf_settings* st);
// Grid of the scene's step: fitted to the domain (clamp on) or to the
// particles' bounding box.
GridDesc fit_grid(const pbf_scene* s);
// Per-step constants of the scene with time step dt (no allocation).
int scene_consts(const pbf_scene* s, float dt, StepConsts& C);
// Stream-ordered allocation of scene buffers from the device's scene pool.
int pool_alloc(void** p, size_t bytes, int device, cudaStream_t st);
void pool_free(void* p, cudaStream_t st);
// Copies a snapshot into the scene on stream `st` (asynchronous).
int restore_on(pbf_scene* s, const pbf_snapshot* snap, cudaStream_t st);
// Device bytes the scene holds (state, step scratch, offsets table).
size_t scene_device_bytes(const pbf_scene* s);
// Cell slots of the grid a scene with these settings and positions steps on.
uint32_t grid_slots_for(const pbf_settings& st, const float* x3, int n);
// Device copy of the scene's rigid bodies, which then step on the device.
int scene_set_rigid(pbf_scene* s, int nbodies, const pbf_rigid_body* bodies);
// Contact shapes of the device rigid bodies: with nshapes > 0 the rigid step
// runs World's contact pipeline (rigid_world.cuh).  Validates the shapes.
int scene_set_contacts(pbf_scene* s, int nshapes, const pbf_rigid_shape* shapes,
                       const pbf_contact_settings* cs);
// The device copy of the rigid bodies, after the scene's queued work.
int scene_read_rigid(pbf_scene* s, pbf_rigid_body* out);
// FluidWorld's post-step on the scene's stream, without waiting: the coupling
// of the step that produced the current state (boundary density, forces and
// torques from zero) and the rigid step of the device bodies under gravity g.
int scene_couple_rigid_async(pbf_scene* s, float dt, const float g[3]);
// The same for a caller that holds the scene's lock and current device.
int scene_couple_rigid_locked(pbf_scene* s, float dt, const float g[3]);

}  // namespace capi
}  // namespace pbf

struct pbf_batch;

namespace pbf {
namespace capi {

// A batch launch of the serving loop: nsteps[k] steps of each scene
// (distinct, unlocked by the caller; one each when nsteps is null),
// asynchronous on the batch's stream.
struct LaunchSpec {
    int nscenes = 0;
    pbf_scene* const* scenes = nullptr;
    const float* dt = nullptr;
    const int* nsteps = nullptr;
    uint32_t* flags_host = nullptr;  // pinned, nscenes words: non-finite flag per scene
    cudaEvent_t start = nullptr;     // recorded before the first step
    cudaEvent_t* sub = nullptr;      // sub[s] recorded after step index s (s < nsub)
    int nsub = 0;
    cudaEvent_t done = nullptr;      // recorded after the launch
    // Between two steps of a scene k with needs_post[k] set, post(ctx, s, k)
    // enqueues its post-step on the scene's stream (the batch holds the
    // scene's lock); the batch waits for it before that scene steps again.
    int (*post)(void* ctx, pbf_scene* s, int k) = nullptr;
    void* post_ctx = nullptr;
    const unsigned char* needs_post = nullptr;
};
int batch_launch(pbf_batch* b, const LaunchSpec& L);
// Step graphs captured, updated in place and instantiated so far.
void batch_counters(const pbf_batch* b, long long* captures, long long* updates,
                    long long* instantiations, long long* direct);
// Grows the batch's scratch for `particles` particles and `scenes` scenes.
int batch_reserve(pbf_batch* b, int particles, int scenes);
size_t batch_bytes(const pbf_batch* b);

}  // namespace capi
}  // namespace pbf
