/*
 * novaphy_pbf.h - C ABI of the GB300 Position Based Fluids step.
 *
 * This is the drop-in boundary for NovaPhy's PBF fluid path.  Each entry point
 * names the reference interface it replaces (paths inside the NovaPhy tree).
 * Plain C: pointers, sizes and POD structs; no C++ or torch types.
 *
 * Conventions
 *   - Host arrays of 3-vectors are packed float[3*n] in particle order, the
 *     layout of std::vector<Eigen::Vector3f> (include/novaphy/fluid/
 *     particle_state.h:16-44).
 *   - Every function returns PBF_OK (0) or a PBF_ERR_* code; the message of
 *     the last failure on the calling thread is pbf_last_error().
 *   - A scene is device-resident particle state plus its scratch; calls on one
 *     scene are serialised by the scene's mutex and ordered on its stream.
 */
#ifndef NOVAPHY_PBF_H
#define NOVAPHY_PBF_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PBF_ABI_VERSION 1

enum pbf_status {
    PBF_OK = 0,
    PBF_ERR_INVALID_ARG = 1, /* bad pointer, size or setting (pybind: ValueError) */
    PBF_ERR_CUDA = 2,        /* CUDA runtime error */
    PBF_ERR_OOM = 3,         /* device allocation failed */
    PBF_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
    PBF_ERR_NO_DEVICE = 5,   /* no CUDA device / extension unusable */
    PBF_ERR_NONFINITE = 6,   /* non-finite value found by pbf_scene_check_finite */
    PBF_ERR_CAPACITY = 7     /* a size exceeds a fixed maximum */
};

/* Field order of PBFSettings (include/novaphy/fluid/pbf_solver.h:13-38),
 * followed by this library's extensions. */
typedef struct pbf_settings {
    float rest_density;      /* rho0 (kg/m^3) */
    float kernel_radius;     /* h (m); the neighbour grid cell is h */
    float particle_radius;   /* domain clamp inset (m) */
    int solver_iterations;   /* Jacobi density iterations */
    float epsilon;           /* CFM relaxation */
    float xsph_viscosity;    /* XSPH coefficient (0 disables) */
    float vorticity_epsilon; /* vorticity confinement strength (0 disables) */
    float corr_delta_q;      /* s_corr delta_q as a fraction of h */
    float corr_k;            /* s_corr k */
    int corr_n;              /* s_corr exponent: 4, anything else means 2 */
    int use_domain_bounds;   /* clamp to [lower+r, upper-r] at commit */
    float domain_lower[3];
    float domain_upper[3];
    /* --- extensions (not in the reference) --- */
    int exact_arithmetic; /* 1 (default): reference operation order with no
                             fused multiply-add and IEEE div/sqrt (bit-exact
                             with the reference); 0: fast path (FMA, rsqrt,
                             approximate division) */
    int hash_compat;      /* 1 (default): reproduce the reference's XOR-hash
                             bucket merging (neighbor_search.cpp:89-97),
                             including double-visited buckets; 0: plain
                             27-cell neighbourhood */
    int boundary_two_way; /* 0 (default): the reference's coupling, in which
                             the boundary pushes the bodies and never the fluid
                             (fluid_world.cpp:68-79); 1: the Akinci boundary
                             also enters the fluid's density constraint (its
                             density, gradient and position correction) in
                             every Jacobi iteration of pbf_scene_step_coupled,
                             so the fluid is held off the bodies.  No
                             counterpart in the reference; single coupled
                             scenes only (batches and servers refuse it). */
    float boundary_friction; /* with boundary_two_way: XSPH-style friction of the
                                fluid against the bodies' surface velocity,
                                v_i += c sum_b psi_b (v_b - v_i) W_ib, before the
                                fluid's own XSPH (0, the default, disables it;
                                set the bodies' velocities with
                                pbf_scene_set_body_velocities) */
} pbf_settings;

/* Field selectors for pbf_scene_read / pbf_scene_write. */
enum pbf_field {
    PBF_FIELD_POSITIONS = 0,  /* float[3n] */
    PBF_FIELD_VELOCITIES = 1, /* float[3n] */
    PBF_FIELD_DENSITIES = 2,  /* float[n]  */
    PBF_FIELD_LAMBDAS = 3     /* float[n]  */
};

typedef struct pbf_scene pbf_scene;

/* Library identity and the last error message of the calling thread. */
const char* pbf_version(void);
const char* pbf_last_error(void);

/* PBFSettings{} defaults (pbf_solver.h:14-27) plus extension defaults
 * (exact_arithmetic = 1, hash_compat = 1). */
int pbf_default_settings(pbf_settings* out);

/* Number of visible CUDA devices (0 on a host without a GPU). */
int pbf_device_count(int* out);

/* Creates a device-resident scene on `device` from host state: x3/v3 are
 * float[3n] (v3 may be NULL for zero velocity), `mass` the particle mass.
 * Replaces constructing ParticleState + PBFSolver
 * (particle_state.cpp:11-20, pbf_solver.cpp:15-16).  n may be 0. */
int pbf_scene_create(int device, const pbf_settings* settings, int n, const float* x3,
                     const float* v3, float mass, pbf_scene** out);
int pbf_scene_destroy(pbf_scene* scene);

/* Settings are re-read every step, as PBFSolver::settings() edits are
 * (pbf_solver.cpp:24-25). */
int pbf_scene_set_settings(pbf_scene* scene, const pbf_settings* settings);
int pbf_scene_get_settings(const pbf_scene* scene, pbf_settings* out);
int pbf_scene_set_gravity(pbf_scene* scene, const float* g3);
int pbf_scene_set_mass(pbf_scene* scene, float mass);
int pbf_scene_num_particles(const pbf_scene* scene, int* out);

/* Replaces the particle state (ParticleState::init, particle_state.cpp:11-20):
 * positions and velocities are set, densities and lambdas zeroed. */
int pbf_scene_reset(pbf_scene* scene, int n, const float* x3, const float* v3);

/* Advances `nsteps` PBF steps of size dt on the device
 * (PBFSolver::step, pbf_solver.cpp:18-127, repeated).  Asynchronous on the
 * scene's stream; pbf_scene_sync waits and reports device-side errors. */
int pbf_scene_step(pbf_scene* scene, float dt, int nsteps);
int pbf_scene_sync(pbf_scene* scene);

/* pbf_scene_step followed by a wait; *ms_out receives the device time of the
 * nsteps steps measured with CUDA events on the scene's stream. */
int pbf_scene_step_timed(pbf_scene* scene, float dt, int nsteps, float* ms_out);

/* Device-resident snapshot of a scene's particle state (positions,
 * velocities, densities, lambdas) plus its settings, gravity and mass: the
 * checkpoint/resume unit.  Restoring and stepping k + m steps is bit-identical
 * to stepping k, snapshotting, restoring and stepping m.  The reference has no
 * counterpart; ParticleState::init (particle_state.cpp:11-20) is its only way
 * to re-seed a state. */
typedef struct pbf_snapshot pbf_snapshot;
int pbf_snapshot_create(pbf_scene* scene, pbf_snapshot** out);
int pbf_snapshot_restore(pbf_scene* scene, const pbf_snapshot* snap);
int pbf_snapshot_destroy(pbf_snapshot* snap);
int pbf_snapshot_num_particles(const pbf_snapshot* snap, int* out);

/* Benchmark loop: nsteps times { restore `seed`; one step }, bracketed by
 * CUDA events on the scene's stream (the step graph is captured before the
 * timed region); *ms_out receives the device time of the whole loop. */
int pbf_scene_replay_timed(pbf_scene* scene, const pbf_snapshot* seed, float dt, int nsteps,
                           float* ms_out);

/* Copies a field to/from host memory (blocking).  Reading replaces the
 * ParticleState vector accessors (python/bindings/bind_fluid.cpp:120-131). */
int pbf_scene_read(pbf_scene* scene, int field, float* host_out);
int pbf_scene_write(pbf_scene* scene, int field, const float* host_in);

/* Device pointer of a field's float4 (x,y,z,pad) or float array, for callers
 * that keep state on the device.  Valid until the scene is reset/destroyed. */
int pbf_scene_device_field(pbf_scene* scene, int field, void** dptr);

/* The CUDA stream (cudaStream_t) the scene's work is ordered on. */
int pbf_scene_stream(pbf_scene* scene, void** stream);

/* Page-locked (pinned) host memory, usable from every device: pbf_scene_read
 * into it is a single DMA, and the host World's array views of the fluid state
 * sit in it.  No counterpart in the reference, whose ParticleState accessors
 * return list copies (python/bindings/bind_fluid.cpp:120-131).  bytes == 0
 * gives NULL; pbf_host_free(NULL) is a no-op. */
int pbf_host_alloc(size_t bytes, void** out);
int pbf_host_free(void* p);

/* Host-array drop-in of PBFSolver::step(ParticleState&, dt, gravity, mass)
 * (include/novaphy/fluid/pbf_solver.h:72, pbf_solver.cpp:18-127): uploads x,
 * v, densities and lambdas, runs one step, downloads them in place.  The
 * scene is resized to n as needed; n == 0 returns immediately like the
 * reference (pbf_solver.cpp:21). */
int pbf_solver_step_host(pbf_scene* scene, int n, float* x3, float* v3, float* densities,
                         float* lambdas, float dt, const float* g3, float mass);

/* ---- Akinci rigid-fluid coupling (FluidWorld, src/fluid/fluid_world.cpp) ---- */

/* Boundary particles (BoundaryParticle, include/novaphy/fluid/boundary.h:21-25):
 * body-frame positions local3[3nb], owning body (-1 = world-owned, local is
 * world), Akinci volume psi. */
int pbf_scene_set_boundary(pbf_scene* scene, int nb, const float* local3, const int* body,
                           const float* psi);

/* Body poses at the start of the next coupled step (World state transforms):
 * positions pos3[3k], unit quaternions quat4[4k] as (w, x, y, z), and which
 * bodies are dynamic (static bodies get no coupling force,
 * fluid_world.cpp:141).  nbodies must cover every body the boundary names. */
int pbf_scene_set_bodies(pbf_scene* scene, int nbodies, const float* pos3, const float* quat4,
                         const int* dynamic);

/* Linear and angular velocities (world frame) of those bodies, for the
 * boundary friction of two-way coupled steps (pbf_settings.boundary_friction):
 * a boundary particle moves with v + w x (x_b - p) of its body, a world-owned
 * one not at all.  Zero until set.  No counterpart in the reference. */
int pbf_scene_set_body_velocities(pbf_scene* scene, int nbodies, const float* lin3,
                                  const float* ang3);

/* The fluid part of FluidWorld::step (fluid_world.cpp:57-81): boundary world
 * positions from the current body poses, one PBF step, boundary density added
 * to the final densities, and the coupling force / torque of every boundary
 * particle accumulated into force3 / torque3 (nbodies * 3 each, in and out)
 * in boundary order, exactly as World::apply_force / apply_torque add them.
 * The rigid step that follows stays with the caller. */
int pbf_scene_step_coupled(pbf_scene* scene, float dt, float* force3, float* torque3);

/* The coupling half of pbf_scene_step_coupled, for a scene whose PBF step ran
 * elsewhere (for instance in a pbf_batch_step with other scenes): boundary
 * world positions from the current body poses, boundary density added to the
 * densities, coupling forces / torques accumulated into force3 / torque3.
 * pbf_scene_step(dt) followed by pbf_scene_couple(dt) equals
 * pbf_scene_step_coupled(dt) bit for bit (the PBF step never reads the
 * boundary).  dt must be the step's time step. */
int pbf_scene_couple(pbf_scene* scene, float dt, float* force3, float* torque3);
/* pbf_scene_couple that also reports the device time (ms) of its three
 * phases in phase_ms[0..2]: boundary world positions, boundary density,
 * coupling forces and torques (fluid_world.cpp:52-85 phase names
 * fluid.boundary.positions, fluid.boundary_density, fluid.coupling.total). */
int pbf_scene_couple_profiled(pbf_scene* scene, float dt, float* force3, float* torque3,
                              float* phase_ms);

/* World positions of the boundary particles used by the last coupled step. */
int pbf_scene_read_boundary(pbf_scene* scene, float* world3);

/* Akinci volumes psi_b = 1 / sum_b' poly6 (boundary.cpp:152-176) of nb boundary
 * particles at world positions world3, computed on `device`. */
int pbf_boundary_volumes(int device, int nb, const float* world3, float kernel_radius,
                         float* psi_out);

/* Finite check of positions and velocities; PBF_ERR_NONFINITE when any
 * component is NaN/Inf. */
int pbf_scene_check_finite(pbf_scene* scene);

/* Cell coordinates floor(x * (1/h)) of the predicted positions of the next
 * step (neighbor_search.cpp:99-105), int[3n] in particle order; for parity. */
int pbf_scene_debug_cells(pbf_scene* scene, float dt, int* cells3);

/* Canonical neighbour sets at the predicted positions of the next step:
 * for particle i, the sorted {j != i : |x*_i - x*_j|^2 < h^2} taken over the
 * grid candidates (pbf_solver.cpp:43-51 restricted to the kernel support).
 * offsets: long long[n+1]; out_idx: int[cap].  Returns the total in *total;
 * pass out_idx = NULL to size. */
int pbf_scene_debug_neighbors(pbf_scene* scene, float dt, long long* offsets, int* out_idx,
                              long long cap, long long* total);

/* Number of phases reported by pbf_scene_step_profiled. */
#define PBF_NUM_PHASES 7

/* Name of a step phase: the reference's PerformanceMonitor scope it maps to
 * (pbf_solver.cpp:29-103), NULL when out of range.  Fused kernels report
 * under the first scope they cover. */
const char* pbf_phase_name(int phase);

/* Runs ONE step without graph replay, with CUDA events between the phases,
 * and returns the device time of each phase (ms) and its kernel launches.
 * phase_ms / launches have PBF_NUM_PHASES entries (launches may be NULL). */
int pbf_scene_step_profiled(pbf_scene* scene, float dt, float* phase_ms, int* launches);

/* One-shot device radix sort of (key, index) pairs with 32-bit keys below
 * 2^key_bits, stable: out_keys/out_vals receive keys in ascending order and
 * the original positions.  Exposed for testing the sort used by the step. */
int pbf_sort_pairs_host(int device, int n, const unsigned* keys, int key_bits,
                        unsigned* out_keys, unsigned* out_vals);

/* Allocation-free cell-key sort.  No counterpart in the reference: it exists
 * for callers that must not allocate device memory while they run (a host
 * framework that owns all device memory through its own budgeted pool, or a
 * latency-bound loop where cudaMalloc/cudaFree could synchronize the device
 * or fail mid-frame).  Same result as pbf_sort_pairs_host, but keys and
 * outputs are DEVICE buffers the caller owns, and the sort's scratch is a
 * fixed static device array (about 4.2 MB held on every GPU that loads the
 * library, until exit), so at most 262,144 keys (PBF_ERR_CAPACITY beyond).
 * The first call on a device looks up the array's address with that device
 * current.  d_keys, d_out_keys and d_out_vals must not overlap (an in-place
 * sort is refused with PBF_ERR_INVALID_ARG).  Calls share the array: calls
 * whose work overlaps on the GPU race and must be serialized.  The call
 * blocks until the sort on `stream` (a cudaStream_t, NULL for the default
 * stream) is done and its status is read back, so it cannot be recorded into
 * a CUDA graph: on a stream under capture it returns PBF_ERR_INVALID_ARG. */
int pbf_sort_pairs_noalloc(int device, int n, const unsigned* d_keys, int key_bits,
                           unsigned* d_out_keys, unsigned* d_out_vals, void* stream);


/* ---- Batches of scenes --------------------------------------------------
 * No counterpart in the reference, which steps one FluidWorld at a time
 * (src/fluid/fluid_world.cpp:49-97, PBFSolver::step at
 * src/fluid/pbf_solver.cpp:18-127).  A batch steps many independent scenes
 * together: one cell-key sort, one reference-key sort and one kernel launch
 * per phase for all of them, with each scene's own settings, gravity, mass,
 * time step and iteration count read from a per-scene table on the device.
 * The scenes keep their state in place; a scene stepped in a batch ends
 * bit for bit where pbf_scene_step would have left it. */
typedef struct pbf_batch pbf_batch;

/* A batch context on `device`; its scratch grows to the largest batch. */
int pbf_batch_create(int device, pbf_batch** out);
int pbf_batch_destroy(pbf_batch* batch);

/* Steps scenes[k] (distinct, on the batch's device) nsteps[k] times with
 * time step dt[k]; nsteps may be NULL for one step each.  Scenes with no
 * particles or no steps are skipped.  Asynchronous: the batch's stream first
 * waits for the scenes' pending work, and later calls on the scenes are
 * ordered after the batch.  Scenes with exact_arithmetic 1 and 0 are stepped
 * as two launches sequences. */
int pbf_batch_step(pbf_batch* batch, int nscenes, pbf_scene* const* scenes, const float* dt,
                   const int* nsteps);

/* pbf_batch_step bracketed by CUDA events on the batch's stream; waits for
 * the end and returns the device time (ms) in *ms_out. */
int pbf_batch_step_timed(pbf_batch* batch, int nscenes, pbf_scene* const* scenes,
                         const float* dt, const int* nsteps, float* ms_out);

/* Restores every scene from seeds[k] and runs one batch step, nsteps times,
 * timed as one region (the seeded step of a benchmark). */
int pbf_batch_replay_timed(pbf_batch* batch, int nscenes, pbf_scene* const* scenes,
                           const pbf_snapshot* const* seeds, const float* dt, int nsteps,
                           float* ms_out);

/* on != 0: run the Jacobi iterations of each batch step as one persistent
 * cooperative launch (a grid sized to stay resident loops over the particles
 * and meets at a bounded grid barrier after every pass) instead of one launch
 * per pass.  Results are identical either way.  Off by default. */
int pbf_batch_set_persistent(pbf_batch* batch, int on);

/* on != 0: autotune each class of batch shape (arithmetic build,
 * particle-count octave, largest iteration count, vorticity).  The first four
 * steps of a class each run one choice of {block size of the neighbour passes
 * 128, 64, 256; persistent Jacobi loop} timed with events on the batch's
 * stream; later steps use the fastest.  Results are identical under every
 * choice.  Decisions are appended to a JSON-lines file keyed by GPU name
 * ($PBF_AUTOTUNE_CACHE, default ~/.cache/novaphy_gb300/autotune.jsonl) and
 * read back when autotuning is switched on.  Off by default. */
int pbf_batch_set_autotune(pbf_batch* batch, int on);

/* Block size and persistent flag the batch's last step ran with. */
int pbf_batch_tuning(const pbf_batch* batch, int* block, int* persistent);

/* Waits for the batch's stream and checks its device status word (a grid
 * barrier that gave up is reported as PBF_ERR_TIMEOUT). */
int pbf_batch_sync(pbf_batch* batch);

/* After a pbf_batch_step of nscenes scenes: out[k] = 1 when a step of
 * scenes[k] committed a non-finite position or velocity, else 0 (waits for
 * the batch).  nscenes must equal the last call's. */
int pbf_batch_nonfinite(pbf_batch* batch, int nscenes, int* out);

/* Device bytes held: by a batch's scratch, and by a scene's resident state
 * plus whatever scratch its own steps have allocated. */
int pbf_batch_device_bytes(const pbf_batch* batch, size_t* out);
int pbf_scene_device_bytes(const pbf_scene* scene, size_t* out);

/* Device bytes per particle of a scene's resident state (x, v, rho, lambda
 * and a staging buffer), the figure an admission budget counts. */
size_t pbf_state_bytes_per_particle(void);


/* ---- Serving loop -------------------------------------------------------
 * No counterpart in the reference (it has no server; each FluidWorld is
 * stepped by its owner, src/fluid/fluid_world.cpp:49).  A server keeps
 * scenes resident on one device and steps them for many clients.  Requests
 * (k steps of one scene, from any thread) are coalesced into batch launches
 * by the server's scheduler, which owns the batch stream: continuous batching,
 * so a request that arrives while launches are in flight joins the next
 * launch, and each scene's steps run in request order.  Scenes are admitted
 * against an HBM budget (resident state plus a grid share, and the batch
 * scratch reserved at creation); a scene that does not fit waits in a FIFO
 * until memory frees up, and one that can never fit is rejected.  A step
 * that commits a non-finite position or velocity fails its scene (its
 * requests fail with PBF_ERR_NONFINITE; a launch that fails fails its
 * scenes with the launch's status); the other scenes are unaffected.
 * A scene's results do not depend on what it was batched with. */
typedef struct pbf_server pbf_server;

typedef struct pbf_server_config {
    size_t hbm_budget_bytes; /* scenes' charged bytes + batch scratch */
    int max_batch_particles; /* particles per launch (the scratch is sized for it) */
    int max_batch_scenes;    /* scenes per launch */
    int max_inflight;        /* launches queued on the GPU ahead of completion, >= 1 */
    int min_step_particles;  /* a launch runs further steps of its scenes with the
                                deepest queues only when each further step holds
                                at least this many particles (and a quarter of
                                the launch's); default 1M */
} pbf_server_config;

enum pbf_scene_state {
    PBF_SCENE_WAITING = 0,  /* queued for admission */
    PBF_SCENE_RESIDENT = 1, /* on the device, served */
    PBF_SCENE_FAILED = 2    /* a step went non-finite; requests fail */
};

enum pbf_request_state { PBF_REQ_PENDING = 0, PBF_REQ_DONE = 1, PBF_REQ_FAILED = 2 };

typedef struct pbf_server_stats {
    long long scenes_resident, scenes_waiting, scenes_rejected, scenes_failed;
    long long requests_submitted, requests_done, requests_failed;
    long long steps_done;     /* scene-steps completed */
    long long particle_steps; /* particles x steps completed */
    long long launches;       /* batch launches */
    long long queue_depth;    /* requests submitted and not finished */
    /* Step latency: from the later of a request's submission and its
     * previous step's completion to this step's completion.  Request
     * latency: submission to last step's completion.  Host clock, ms;
     * percentiles of a fixed-memory log histogram, within 0.25 % of exact. */
    double step_ms_p50, step_ms_p99;
    double request_ms_p50, request_ms_p99;
    double particle_steps_per_s; /* first submission to last completion */
    double mean_launch_scenes, mean_launch_particles;
    size_t hbm_bytes_charged;       /* admitted scenes */
    size_t hbm_bytes_scratch;       /* batch scratch */
    size_t state_bytes_per_particle; /* resident bytes charged per particle */
    size_t grid_bytes_per_slot;      /* bytes charged per cell slot of a scene's grid */
    double issue_ms_mean;            /* host time to issue one launch */
    long long graph_captures;        /* step graphs captured (new launch shapes) */
    long long graph_updates;         /* ... applied to the instantiated graph in place */
    long long graph_instantiations;  /* ... instantiated anew */
    long long launches_direct;       /* step launches issued without a graph (a
                                        shape is captured when seen twice in a row) */
    double post_ms_mean;             /* part of issue_ms_mean spent enqueueing the
                                        coupled scenes' coupling and rigid step */
} pbf_server_stats;

/* Defaults: 120 GB budget, 16M particles and 1024 scenes per launch, 2
 * launches in flight. */
int pbf_server_default_config(pbf_server_config* out);
int pbf_server_create(int device, const pbf_server_config* config, pbf_server** out);
/* Stops the scheduler after the launches in flight, frees every scene. */
int pbf_server_destroy(pbf_server* server);

/* Opens a scene (state copied from the host arrays; gravity3 may be NULL for
 * the World default).  *state_out (may be NULL) is PBF_SCENE_RESIDENT or
 * PBF_SCENE_WAITING.  PBF_ERR_CAPACITY when the scene can never fit. */
int pbf_server_open_scene(pbf_server* server, const pbf_settings* settings, int n,
                          const float* x3, const float* v3, float mass, const float* gravity3,
                          long long* scene_id, int* state_out);
/* Waits for the scene's requests, then frees it and admits waiting scenes. */
int pbf_server_close_scene(pbf_server* server, long long scene_id);
/* Queues nsteps steps of the scene with time step dt; returns at once. */
int pbf_server_submit(pbf_server* server, long long scene_id, float dt, int nsteps,
                      long long* request_id);
/* Waits up to timeout_s seconds (< 0: no limit) for a request; *state_out is
 * its pbf_request_state.  PBF_ERR_TIMEOUT if still pending; a failed request
 * returns its failure status, with the reason in pbf_last_error().  The
 * server keeps the records of the latest 65536 finished requests; waiting on
 * an older finished request returns PBF_ERR_INVALID_ARG. */
int pbf_server_wait(pbf_server* server, long long request_id, double timeout_s, int* state_out);
/* A rigid body of a served coupled scene: the state World's semi-implicit
 * Euler integrates (src/dynamics/integrator.cpp), which the server runs on
 * the device, for free bodies or, with contact shapes
 * (pbf_server_open_coupled_scene_contacts), through World's contact pipeline.
 * inv_mass 0 marks a static body; inv_inertia is RigidBody::inv_inertia,
 * row-major. */
typedef struct pbf_rigid_body {
    float pos[3];
    float quat[4]; /* w, x, y, z */
    float lin_vel[3];
    float ang_vel[3];
    float inv_mass;
    float inv_inertia[9];
} pbf_rigid_body;

/* A collision shape of a served coupled scene's rigid contacts
 * (CollisionShape, include/novaphy/collision/shape.h: make_sphere,
 * make_plane, ModelBuilder::add_ground_plane).  Spheres and planes. */
#define PBF_SHAPE_SPHERE 0
#define PBF_SHAPE_PLANE 1
typedef struct pbf_rigid_shape {
    int type;           /* PBF_SHAPE_* */
    int body;           /* sphere: its body (-1: fixed in the world); plane: -1 */
    float radius;       /* sphere */
    float local_pos[3]; /* sphere: centre in the body frame (local_transform.position) */
    float normal[3];    /* plane: unit normal (make_plane normalises it) */
    float offset;       /* plane: normal . x = offset */
    float friction;
    float restitution;
} pbf_rigid_shape;

/* The contact solve's SolverSettings (include/novaphy/sim/world.h). */
typedef struct pbf_contact_settings {
    int velocity_iterations; /* 30 */
    float baumgarte;         /* 0.3 */
    float slop;              /* 0.005 */
    int warm_starting;       /* 1 */
} pbf_contact_settings;

/* Opens a coupled scene: the fluid of pbf_server_open_scene plus nb Akinci
 * boundary particles (pbf_scene_set_boundary layout; psi from
 * pbf_boundary_volumes) owned by nbodies rigid bodies.  Each served step of
 * it is FluidWorld::step (src/fluid/fluid_world.cpp:46-99): the PBF step,
 * batched with the other scenes; the coupling (pbf_scene_couple); then the
 * rigid step of the bodies under gravity and the coupling forces (World's
 * semi-implicit Euler of free bodies, run on the device with the same float
 * operations), before the scene's next step.  The scene is charged its own
 * step scratch too, which the coupling uses. */
int pbf_server_open_coupled_scene(pbf_server* server, const pbf_settings* settings, int n,
                                  const float* x3, const float* v3, float mass,
                                  const float* gravity3, int nb, const float* local3,
                                  const int* body, const float* psi, int nbodies,
                                  const pbf_rigid_body* bodies, long long* scene_id,
                                  int* state_out);

/* pbf_server_open_coupled_scene whose bodies also collide: after each step's
 * coupling the server runs World's rigid pipeline on the device
 * (src/sim/world.cpp:30-182 with sleep off: symplectic Euler, shape boxes,
 * broad phase, sphere-sphere and sphere-plane contacts, the warm-started
 * sequential-impulse solve of src/dynamics/free_body_solver.cpp, position
 * update) with the float operations of the host World, so the bodies follow
 * FluidWorld::step bit for bit.  Up to 16 shapes and 16 bodies; a shape
 * other than a sphere or a plane, or one naming a missing body, is
 * PBF_ERR_INVALID_ARG. */
int pbf_server_open_coupled_scene_contacts(
    pbf_server* server, const pbf_settings* settings, int n, const float* x3, const float* v3,
    float mass, const float* gravity3, int nb, const float* local3, const int* body,
    const float* psi, int nbodies, const pbf_rigid_body* bodies, int nshapes,
    const pbf_rigid_shape* shapes, const pbf_contact_settings* contact_settings,
    long long* scene_id, int* state_out);

/* The bodies of a coupled scene after its completed steps (waits until the
 * scene has no pending request). */
int pbf_server_read_bodies(pbf_server* server, long long scene_id, pbf_rigid_body* out);

/* Waits until the scene has no pending request, then reads a field
 * (pbf_scene_read layout). */
int pbf_server_read(pbf_server* server, long long scene_id, int field, float* host_out);
int pbf_server_scene_state(pbf_server* server, long long scene_id, int* state_out);
int pbf_server_get_stats(pbf_server* server, pbf_server_stats* out);
/* Clears latency samples and counters of completed work. */
int pbf_server_reset_stats(pbf_server* server);

#ifdef __cplusplus
}
#endif

#endif /* NOVAPHY_PBF_H */
