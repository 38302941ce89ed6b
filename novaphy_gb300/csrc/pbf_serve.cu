// Serving loop (include/novaphy_pbf.h, "Serving loop"): device-resident
// scenes stepped for many clients by a scheduler that coalesces pending
// requests into batch launches on one stream.
//
// Scheduling.  Every resident scene has a FIFO of requests; its issuable
// request is the first one with steps not yet issued.  A launch takes one
// step of every scene with an issuable request, oldest request first, up to
// the per-launch particle and scene caps.  A heavily loaded launch takes
// further steps of the scenes with the deepest queues (up to kMaxSubSteps
// each; launch_plan.hpp): the batch runs them as consecutive steps, so deep
// queues drain at several steps per launch instead of one.  Up to
// max_inflight launches are queued on the batch stream; while they run, the
// scheduler builds the next one from whatever is pending then (continuous
// batching), and a scene can be in several queued launches at once because
// the stream orders them.
// A second thread waits on the oldest launch's event and retires its steps,
// which frees its slot for the next launch.
//
// Coupled scenes (FluidWorld with rigid bodies) step like the others: right
// after a launch is issued, the issue thread enqueues on each coupled scene's
// stream the coupling of its last step and the rigid step of its bodies,
// which live on the device (between two steps of one launch, the batch does
// the same and waits for it).  The next launch waits for the scene's stream,
// so the device runs step, coupling, rigid step, next step in order with no
// host round trip.
//
// Admission.  A scene is charged state_bytes * n + grid_bytes * slots of its
// grid (the share of the batch's offset table a launch holding it can use).
// The batch scratch for max_batch_particles is reserved at creation.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <functional>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "latency_hist.hpp"
#include "launch_plan.hpp"
#include "pbf_internal.cuh"
#include "rigid_step.hpp"

using namespace pbf;
using namespace pbf::capi;

namespace {

constexpr size_t kGridBytesPerSlot = 13;  // offset word, alias byte, moved and lambda words
// Records of finished requests kept for pbf_server_wait; older ones are
// dropped, so a long-running server holds bounded host memory.
constexpr size_t kFinishedKept = (size_t)1 << 16;
// Device bytes per boundary particle of a coupled scene: local, world and force
// float4s, body index, query cell and classification row, boundary index.
constexpr size_t kBoundaryBytes = 256;

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct SceneRec {
    long long id = 0;
    pbf_scene* s = nullptr;
    int state = PBF_SCENE_WAITING;
    int n = 0;
    size_t charge = 0;
    bool busy = false;  // device copy being made or read outside the lock
    // Host copy while waiting for admission.
    pbf_settings settings{};
    std::vector<float> x, v;
    float mass = 0.0f;
    float gravity[3] = {0.0f, -9.81f, 0.0f};
    std::deque<long long> reqs;  // FIFO
    int inflight = 0;            // steps issued, not completed
    std::string why;             // why the scene failed
    int code = PBF_OK;           // and the status its requests fail with
    // Coupled scenes (FluidWorld): Akinci boundary owned by rigid bodies that
    // the host rigid step advances after each step of the scene.
    bool coupled = false;
    std::vector<float> local, psi;  // until the device copy is made
    std::vector<int> body;
    std::vector<pbf_rigid_body> bodies;  // until the device copy is made
    std::vector<pbf_rigid_shape> shapes; // contact shapes of the bodies (none: free bodies)
    pbf_contact_settings cset{30, 0.3f, 0.005f, 1};
};

struct ReqRec {
    long long id = 0, scene = 0;
    float dt = 0.0f;
    int nsteps = 0, issued = 0, done = 0;
    int state = PBF_REQ_PENDING;
    double t_submit = 0.0, t_prev = 0.0;
    std::string why;  // why the request failed
    int code = PBF_OK;
};

constexpr int kMaxSubSteps = 16;  // steps of one scene in one launch

struct LaunchItem {
    long long scene = 0;
    int steps = 0;
    std::vector<std::pair<long long, int>> reqs;  // (request, steps taken from it), in order
};

struct Launch {
    int slot = 0;
    std::vector<LaunchItem> items;
    long long particles = 0;  // particles of the launch's scenes
    long long work = 0;       // particle-steps
    int max_steps = 0;
};

}  // namespace

struct pbf_server {
    int device = 0;
    pbf_server_config cfg{};
    pbf_batch* batch = nullptr;
    size_t scratch = 0;

    std::mutex mu;
    std::condition_variable cv_work, cv_retire, cv_done;
    bool stop = false;
    std::thread issuer, retirer;

    std::map<long long, SceneRec> scenes;
    std::deque<long long> admit_queue;
    std::unordered_map<long long, ReqRec> reqs;
    std::deque<long long> finished;  // ids of finished requests, oldest first
    long long next_scene = 1, next_req = 1;
    size_t charged = 0;

    std::deque<Launch> inflight;
    std::vector<cudaEvent_t> events;              // per slot: end of the launch
    std::vector<cudaEvent_t> ev_start, ev_sub;    // per slot: timing of its steps
    uint32_t* flags = nullptr;  // pinned, max_inflight x max_batch_scenes
    int next_slot = 0;

    // statistics
    long long rejected = 0, failed_scenes = 0, submitted = 0, done_reqs = 0, failed_reqs = 0;
    long long steps_done = 0, particle_steps = 0, launches = 0, launch_scenes = 0,
              launch_particles = 0;
    double t_first = -1.0, t_last = 0.0;
    double issue_ms = 0.0;  // host time spent issuing launches
    double post_ms = 0.0;   // ... of which enqueueing coupled scenes' post-steps
    pbf_stats::LatencyHist step_ms, req_ms;
};

namespace {

// Charged bytes of a scene with n particles on a grid of `slots` cells.
size_t charge_of(int n, uint32_t slots) {
    return (size_t)n * kStateBytesPerParticle + (size_t)slots * kGridBytesPerSlot;
}

// Records that request `id` reached a final state, dropping the oldest
// finished records beyond kFinishedKept.
void note_finished(pbf_server* sv, long long id) {
    sv->finished.push_back(id);
    while (sv->finished.size() > kFinishedKept) {
        sv->reqs.erase(sv->finished.front());
        sv->finished.pop_front();
    }
}

void fail_request(pbf_server* sv, ReqRec& r, const std::string& why, int code) {
    if (r.state != PBF_REQ_PENDING) return;
    r.state = PBF_REQ_FAILED;
    r.why = why;
    r.code = code;
    ++sv->failed_reqs;
    note_finished(sv, r.id);
}

// The request record of id, or nullptr when it does not exist (any more).
ReqRec* find_req(pbf_server* sv, long long id) {
    auto it = sv->reqs.find(id);
    return it == sv->reqs.end() ? nullptr : &it->second;
}

bool req_pending(pbf_server* sv, long long id) {
    const ReqRec* r = find_req(sv, id);
    return r && r->state == PBF_REQ_PENDING;
}

// code: PBF_ERR_NONFINITE for a non-finite state, else the failing call's.
void fail_scene(pbf_server* sv, SceneRec& sc, const std::string& why, int code) {
    if (sc.state == PBF_SCENE_FAILED) return;
    sc.state = PBF_SCENE_FAILED;
    sc.why = why;
    sc.code = code;
    ++sv->failed_scenes;
    // Collect first: failing a request may drop older finished records.
    const std::vector<long long> ids(sc.reqs.begin(), sc.reqs.end());
    sc.reqs.clear();
    for (long long rid : ids)
        if (ReqRec* r = find_req(sv, rid)) fail_request(sv, *r, "its scene failed: " + why, code);
}

void credit_step(pbf_server* sv, SceneRec& sc, ReqRec& r, double t);

// Marks completed steps of a finished launch; called with the lock held.  A
// coupled scene's step is credited when its PBF step completes; its coupling
// and rigid step follow on the scene's stream, ahead of any later work there.
// t_step[s] is the completion time of the launch's step index s.
void complete_launch(pbf_server* sv, const Launch& L, const std::vector<double>& t_step) {
    const uint32_t* fl = sv->flags + (size_t)L.slot * sv->cfg.max_batch_scenes;
    for (size_t k = 0; k < L.items.size(); ++k) {
        const LaunchItem& it = L.items[k];
        auto sit = sv->scenes.find(it.scene);
        if (sit == sv->scenes.end()) continue;
        SceneRec& sc = sit->second;
        sc.inflight -= it.steps;
        if (fl[k])
            fail_scene(sv, sc, "a step committed a non-finite position or velocity",
                       PBF_ERR_NONFINITE);
        size_t s = 0;
        for (const auto& rq : it.reqs)
            for (int j = 0; j < rq.second; ++j, ++s) {
                ReqRec* r = find_req(sv, rq.first);
                if (r && r->state == PBF_REQ_PENDING)
                    credit_step(sv, sc, *r, t_step[std::min(s, t_step.size() - 1)]);
            }
    }
}

// Counts one completed step of request r of scene sc at time t.
void credit_step(pbf_server* sv, SceneRec& sc, ReqRec& r, double t) {
    ++r.done;
    ++sv->steps_done;
    sv->particle_steps += sc.n;
    sv->step_ms.add(t - r.t_prev);
    r.t_prev = t;
    sv->t_last = t;
    if (r.done == r.nsteps) {
        r.state = PBF_REQ_DONE;
        ++sv->done_reqs;
        sv->req_ms.add(t - r.t_submit);
        if (!sc.reqs.empty() && sc.reqs.front() == r.id) sc.reqs.pop_front();
        note_finished(sv, r.id);  // last: may drop the record r refers to
    }
}

// Builds the next launch from issuable requests; called with the lock held.
// A coupled scene of a launch: its index among the launch's items and its
// gravity.
struct CoupledItem {
    int item;
    float g[3];
};

// The first request of sc with steps not yet issued, or null.
ReqRec* issuable(pbf_server* sv, SceneRec& sc) {
    for (long long rid : sc.reqs) {
        ReqRec* r = find_req(sv, rid);
        if (r && r->state == PBF_REQ_PENDING && r->issued < r->nsteps) return r;
    }
    return nullptr;
}

long long unissued_steps(pbf_server* sv, const SceneRec& sc) {
    long long n = 0;
    for (long long rid : sc.reqs) {
        const ReqRec* r = find_req(sv, rid);
        if (r && r->state == PBF_REQ_PENDING) n += r->nsteps - r->issued;
    }
    return n;
}

bool build_launch(pbf_server* sv, Launch& L, std::vector<pbf_scene*>& ptrs,
                  std::vector<float>& dts, std::vector<int>& nsteps,
                  std::vector<unsigned char>& needs_post, std::vector<CoupledItem>& coupled) {
    struct Cand {
        double t;
        SceneRec* sc;
        ReqRec* r;
    };
    std::vector<Cand> cand;
    for (auto& kv : sv->scenes) {
        SceneRec& sc = kv.second;
        if (sc.state != PBF_SCENE_RESIDENT || !sc.s || sc.busy) continue;
        for (long long rid : sc.reqs) {
            ReqRec* r = find_req(sv, rid);
            if (r && r->state == PBF_REQ_PENDING && r->issued < r->nsteps) {
                cand.push_back({r->t_submit, &sc, r});
                break;
            }
        }
    }
    if (cand.empty()) return false;
    std::sort(cand.begin(), cand.end(), [](const Cand& a, const Cand& b) { return a.t < b.t; });
    L.items.clear();
    L.particles = L.work = 0;
    L.max_steps = 0;
    ptrs.clear();
    dts.clear();
    nsteps.clear();
    needs_post.clear();
    coupled.clear();
    std::vector<SceneRec*> recs;
    const long long cap = sv->cfg.max_batch_particles;
    for (const Cand& c : cand) {
        if ((int)L.items.size() >= sv->cfg.max_batch_scenes) break;
        if (!L.items.empty() && L.particles + c.sc->n > cap) continue;
        if (c.sc->coupled)
            coupled.push_back({(int)L.items.size(), {c.sc->gravity[0], c.sc->gravity[1],
                                                     c.sc->gravity[2]}});
        LaunchItem it;
        it.scene = c.sc->id;
        it.steps = 1;
        it.reqs.push_back({c.r->id, 1});
        L.items.push_back(std::move(it));
        L.particles += c.sc->n;
        ptrs.push_back(c.sc->s);
        dts.push_back(c.r->dt);
        needs_post.push_back(c.sc->coupled ? 1 : 0);
        recs.push_back(c.sc);
        ++c.r->issued;
        ++c.sc->inflight;
    }
    L.work = L.particles;
    // Further steps of the deepest queues (launch_plan.hpp); a scene's further
    // steps keep its first step's dt.
    std::vector<pbf_plan::PlanItem> plan(L.items.size());
    for (size_t k = 0; k < L.items.size(); ++k) {
        plan[k].n = recs[k]->n;
        plan[k].depth = unissued_steps(sv, *recs[k]);
        long long avail = 0;
        for (long long rid : recs[k]->reqs) {
            const ReqRec* r = find_req(sv, rid);
            if (!r || r->state != PBF_REQ_PENDING || r->issued >= r->nsteps) continue;
            if (r->dt != dts[k]) break;
            avail += r->nsteps - r->issued;
            if (avail >= kMaxSubSteps) break;
        }
        plan[k].avail = (int)std::min<long long>(avail, kMaxSubSteps);
    }
    const std::vector<int> steps = pbf_plan::plan_steps(
        plan, cap, std::max(sv->cfg.min_step_particles, 0), kMaxSubSteps);
    for (size_t k = 0; k < L.items.size(); ++k) {
        LaunchItem& it = L.items[k];
        for (int j = 1; j < steps[k]; ++j) {
            ReqRec* r = issuable(sv, *recs[k]);
            ++r->issued;
            ++recs[k]->inflight;
            ++it.steps;
            if (it.reqs.back().first == r->id) ++it.reqs.back().second;
            else it.reqs.push_back({r->id, 1});
            L.work += recs[k]->n;
        }
    }
    for (const LaunchItem& it : L.items) {
        nsteps.push_back(it.steps);
        L.max_steps = std::max(L.max_steps, it.steps);
    }
    return !L.items.empty();
}

// Between two steps of a coupled scene inside one launch: its coupling and
// rigid step (the batch holds the scene's lock and device).
struct PostCtx {
    const std::vector<float>* dts;
    const std::vector<CoupledItem>* coupled;
    std::vector<int> slot_of;  // item -> index in coupled
};

int post_between_steps(void* ctx, pbf_scene* s, int k) {
    const PostCtx* c = static_cast<const PostCtx*>(ctx);
    const CoupledItem& ci = (*c->coupled)[(size_t)c->slot_of[(size_t)k]];
    return scene_couple_rigid_locked(s, (*c->dts)[(size_t)k], ci.g);
}

// Host threads that enqueue the coupled scenes' post-steps of one launch
// (each scene has its own stream and lock, so they proceed in parallel).
constexpr size_t kPostThreads = 8;

void enqueue_posts(pbf_server* sv, const std::vector<CoupledItem>& coupled,
                   const std::vector<pbf_scene*>& ptrs, const std::vector<float>& dts,
                   std::vector<std::pair<int, std::string>>& failed) {
    std::mutex fmu;
    auto one = [&](const CoupledItem& c) {
        if (scene_couple_rigid_async(ptrs[(size_t)c.item], dts[(size_t)c.item], c.g)) {
            std::lock_guard<std::mutex> lk(fmu);
            failed.push_back({c.item, pbf_last_error()});
        }
    };
    const size_t nt = std::min(kPostThreads, coupled.size() / 8);
    if (nt <= 1) {
        for (const CoupledItem& c : coupled) one(c);
        return;
    }
    std::atomic<size_t> next{0};
    std::vector<std::thread> pool;
    pool.reserve(nt);
    for (size_t t = 0; t < nt; ++t)
        pool.emplace_back([&] {
            cudaSetDevice(sv->device);
            for (size_t i; (i = next.fetch_add(1)) < coupled.size();) one(coupled[i]);
        });
    for (auto& t : pool) t.join();
}

// Issues launches while slots are free and requests are pending.
void issue_main(pbf_server* sv) {
    cudaSetDevice(sv->device);
    std::vector<pbf_scene*> ptrs;
    std::vector<float> dts;
    std::vector<int> nsteps;
    std::vector<unsigned char> needs_post;
    std::vector<CoupledItem> coupled;
    std::unique_lock<std::mutex> lk(sv->mu);
    for (;;) {
        if (sv->stop) break;
        Launch L;
        if ((int)sv->inflight.size() >= sv->cfg.max_inflight ||
            !build_launch(sv, L, ptrs, dts, nsteps, needs_post, coupled)) {
            sv->cv_work.wait(lk);
            continue;
        }
        L.slot = sv->next_slot;
        sv->next_slot = (sv->next_slot + 1) % sv->cfg.max_inflight;
        uint32_t* fl = sv->flags + (size_t)L.slot * sv->cfg.max_batch_scenes;
        lk.unlock();
        const double t_issue = now_ms();
        PostCtx pctx;
        pctx.dts = &dts;
        pctx.coupled = &coupled;
        pctx.slot_of.assign(ptrs.size(), -1);
        for (size_t c = 0; c < coupled.size(); ++c) pctx.slot_of[(size_t)coupled[c].item] = (int)c;
        LaunchSpec spec;
        spec.nscenes = (int)ptrs.size();
        spec.scenes = ptrs.data();
        spec.dt = dts.data();
        spec.nsteps = nsteps.data();
        spec.flags_host = fl;
        spec.start = sv->ev_start[(size_t)L.slot];
        spec.sub = &sv->ev_sub[(size_t)L.slot * kMaxSubSteps];
        spec.nsub = kMaxSubSteps;
        spec.done = sv->events[(size_t)L.slot];
        spec.post = post_between_steps;
        spec.post_ctx = &pctx;
        spec.needs_post = needs_post.data();
        const int rc = batch_launch(sv->batch, spec);
        // FluidWorld's post-step of the coupled scenes, enqueued before the
        // next launch is issued (scenes in flight are not closed).
        std::vector<std::pair<int, std::string>> post_failed;
        const double t_post = now_ms();
        if (!rc) enqueue_posts(sv, coupled, ptrs, dts, post_failed);
        const double t_end = now_ms();
        const double issued = t_end - t_issue;
        lk.lock();
        for (const auto& pf : post_failed) {
            auto sit = sv->scenes.find(L.items[(size_t)pf.first].scene);
            if (sit != sv->scenes.end())
                fail_scene(sv, sit->second, "the coupling failed: " + pf.second, PBF_ERR_CUDA);
        }
        sv->issue_ms += issued;
        sv->post_ms += t_end - t_post;
        ++sv->launches;
        sv->launch_scenes += (long long)L.items.size();
        sv->launch_particles += L.particles;
        if (rc) {
            // The launch did not run: its scenes cannot be trusted.
            const std::string why = std::string("a batch launch failed: ") + pbf_last_error();
            for (auto& it : L.items) {
                auto sit = sv->scenes.find(it.scene);
                if (sit == sv->scenes.end()) continue;
                sit->second.inflight -= it.steps;
                fail_scene(sv, sit->second, why, rc);
            }
            sv->next_slot = L.slot;  // the slot was not used
            sv->cv_done.notify_all();
        } else {
            sv->inflight.push_back(std::move(L));
            sv->cv_retire.notify_one();
        }
    }
}

// Waits for the oldest launch and retires its steps.
void retire_main(pbf_server* sv) {
    cudaSetDevice(sv->device);
    std::unique_lock<std::mutex> lk(sv->mu);
    for (;;) {
        sv->cv_retire.wait(lk, [&] { return !sv->inflight.empty() || sv->stop; });
        if (sv->inflight.empty()) {
            if (sv->stop) break;
            continue;
        }
        const int slot = sv->inflight.front().slot;
        const int max_steps = sv->inflight.front().max_steps;
        lk.unlock();
        const cudaError_t e = cudaEventSynchronize(sv->events[slot]);
        const double t = now_ms();
        // Completion time of each step index: the host time at which the end
        // of the launch was seen, less the device time from that step's end
        // to the launch's last step.
        std::vector<double> t_step((size_t)std::max(max_steps, 1), t);
        if (e == cudaSuccess && max_steps > 1) {
            float ms[kMaxSubSteps];
            bool ok = true;
            for (int s = 0; s < max_steps && ok; ++s)
                ok = cudaEventElapsedTime(&ms[s], sv->ev_start[(size_t)slot],
                                          sv->ev_sub[(size_t)slot * kMaxSubSteps + s]) == cudaSuccess;
            if (ok)
                for (int s = 0; s < max_steps; ++s)
                    t_step[(size_t)s] = t - (double)(ms[max_steps - 1] - ms[s]);
            else
                cudaGetLastError();
        }
        lk.lock();
        Launch L = std::move(sv->inflight.front());
        if (e != cudaSuccess) {
            const std::string why =
                std::string("a batch launch did not complete: ") + cudaGetErrorString(e);
            for (auto& it : L.items) {
                auto sit = sv->scenes.find(it.scene);
                if (sit == sv->scenes.end()) continue;
                sit->second.inflight -= it.steps;
                fail_scene(sv, sit->second, why, PBF_ERR_CUDA);
            }
        } else {
            complete_launch(sv, L, t_step);
        }
        sv->inflight.pop_front();
        sv->cv_work.notify_one();
        sv->cv_done.notify_all();
    }
}

// Creates the device copy of an admitted scene (outside the lock).
int materialize(pbf_server* sv, SceneRec& rec) {
    pbf_scene* s = nullptr;
    int rc = pbf_scene_create(sv->device, &rec.settings, rec.n, rec.x.data(),
                              rec.v.empty() ? nullptr : rec.v.data(), rec.mass, &s);
    if (rc) return rc;
    rc = pbf_scene_set_gravity(s, rec.gravity);
    if (rc) {
        pbf_scene_destroy(s);
        return rc;
    }
    if (rec.coupled) {
        const int nb = (int)rec.body.size(), nbodies = (int)rec.bodies.size();
        rc = pbf_scene_set_boundary(s, nb, rec.local.data(), rec.body.data(), rec.psi.data());
        if (!rc && nbodies > 0) {
            std::vector<float> pos((size_t)3 * nbodies), quat((size_t)4 * nbodies);
            std::vector<int> dyn((size_t)nbodies);
            for (int k = 0; k < nbodies; ++k) {
                const pbf_rigid_body& b = rec.bodies[(size_t)k];
                for (int d = 0; d < 3; ++d) pos[3 * k + d] = b.pos[d];
                for (int d = 0; d < 4; ++d) quat[4 * k + d] = b.quat[d];
                dyn[(size_t)k] = b.inv_mass > 0.0f ? 1 : 0;
            }
            rc = pbf_scene_set_bodies(s, nbodies, pos.data(), quat.data(), dyn.data());
        }
        if (!rc) rc = scene_set_rigid(s, nbodies, rec.bodies.data());
        if (!rc && !rec.shapes.empty())
            rc = scene_set_contacts(s, (int)rec.shapes.size(), rec.shapes.data(), &rec.cset);
        if (rc) {
            pbf_scene_destroy(s);
            return rc;
        }
        rec.local.clear();
        rec.psi.clear();
        rec.body.clear();
    }
    // The scene keeps its own stream: launches order themselves against it
    // with events, and client threads (reads, closes) never put work on the
    // batch stream, which the scheduler may be capturing into a graph.
    rec.s = s;
    return PBF_OK;
}

// Admits waiting scenes in FIFO order while they fit; the caller holds the
// lock, which is released around device allocation.
void admit_waiting(pbf_server* sv, std::unique_lock<std::mutex>& lk) {
    while (!sv->admit_queue.empty()) {
        const long long id = sv->admit_queue.front();
        auto it = sv->scenes.find(id);
        if (it == sv->scenes.end()) {
            sv->admit_queue.pop_front();
            continue;
        }
        SceneRec& rec = it->second;
        if (sv->charged + rec.charge + sv->scratch > sv->cfg.hbm_budget_bytes) break;
        sv->admit_queue.pop_front();
        sv->charged += rec.charge;
        rec.busy = true;
        rec.state = PBF_SCENE_RESIDENT;
        lk.unlock();
        const int rc = materialize(sv, rec);
        lk.lock();
        rec.busy = false;
        sv->cv_done.notify_all();
        rec.x.clear();
        rec.x.shrink_to_fit();
        rec.v.clear();
        rec.v.shrink_to_fit();
        if (rc) fail_scene(sv, rec, std::string("its device copy failed: ") + pbf_last_error(), rc);
        sv->cv_work.notify_one();
        sv->cv_done.notify_all();
    }
}

int check_server(pbf_server* sv) {
    if (!sv) return fail(PBF_ERR_INVALID_ARG, "server is NULL");
    return PBF_OK;
}

}  // namespace

extern "C" {

int pbf_server_default_config(pbf_server_config* out) {
    if (!out) return fail(PBF_ERR_INVALID_ARG, "out is NULL");
    out->hbm_budget_bytes = (size_t)120 << 30;
    out->max_batch_particles = 16 << 20;
    out->max_batch_scenes = 1024;
    out->max_inflight = 2;
    out->min_step_particles = 1 << 20;
    return PBF_OK;
}

int pbf_server_create(int device, const pbf_server_config* cfg, pbf_server** out) {
    if (!cfg || !out) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (cfg->max_batch_particles < 1 || cfg->max_batch_scenes < 1 || cfg->max_inflight < 1 ||
        cfg->max_inflight > 16)
        return fail(PBF_ERR_INVALID_ARG,
                    "max_batch_particles, max_batch_scenes >= 1 and max_inflight in [1, 16]");
    pbf_batch* b = nullptr;
    int rc = pbf_batch_create(device, &b);
    if (rc) return rc;
    std::unique_ptr<pbf_server> sv(new pbf_server());
    sv->device = device;
    sv->cfg = *cfg;
    sv->batch = b;
    {
        DeviceGuard dg(device);
        rc = batch_reserve(b, cfg->max_batch_particles, cfg->max_batch_scenes);
        if (!rc) {
            sv->scratch = batch_bytes(b);
            if (sv->scratch > cfg->hbm_budget_bytes)
                rc = fail(PBF_ERR_CAPACITY, "the batch scratch alone exceeds the HBM budget");
        }
        sv->events.assign((size_t)cfg->max_inflight, nullptr);
        for (auto& e : sv->events)
            if (!rc && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
                rc = fail(PBF_ERR_CUDA, "cudaEventCreate");
        sv->ev_start.assign((size_t)cfg->max_inflight, nullptr);
        sv->ev_sub.assign((size_t)cfg->max_inflight * kMaxSubSteps, nullptr);
        for (auto* v : {&sv->ev_start, &sv->ev_sub})
            for (auto& e : *v)
                if (!rc && cudaEventCreate(&e) != cudaSuccess)
                    rc = fail(PBF_ERR_CUDA, "cudaEventCreate");
        if (!rc && cudaMallocHost(&sv->flags, (size_t)cfg->max_inflight * cfg->max_batch_scenes *
                                                  sizeof(uint32_t)) != cudaSuccess)
            rc = fail(PBF_ERR_OOM, "pinned flags");
    }
    if (rc) {
        for (auto* v : {&sv->events, &sv->ev_start, &sv->ev_sub})
            for (auto e : *v)
                if (e) cudaEventDestroy(e);
        if (sv->flags) cudaFreeHost(sv->flags);
        pbf_batch_destroy(b);
        return rc;
    }
    pbf_server* p = sv.release();
    p->issuer = std::thread(issue_main, p);
    p->retirer = std::thread(retire_main, p);
    *out = p;
    return PBF_OK;
}

int pbf_server_destroy(pbf_server* sv) {
    if (!sv) return PBF_OK;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cv_work.notify_all();
    if (sv->issuer.joinable()) sv->issuer.join();
    sv->cv_retire.notify_all();  // the retirer drains the launches in flight, then stops
    if (sv->retirer.joinable()) sv->retirer.join();
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        std::vector<long long> pending;
        for (auto& kv : sv->reqs)
            if (kv.second.state == PBF_REQ_PENDING) pending.push_back(kv.first);
        for (long long rid : pending)
            if (ReqRec* r = find_req(sv, rid)) fail_request(sv, *r, "the server stopped", PBF_ERR_INVALID_ARG);
    }
    sv->cv_done.notify_all();
    {
        DeviceGuard dg(sv->device);
        for (auto& kv : sv->scenes)
            if (kv.second.s) pbf_scene_destroy(kv.second.s);
        sv->scenes.clear();
        for (auto* v : {&sv->events, &sv->ev_start, &sv->ev_sub})
            for (auto e : *v)
                if (e) cudaEventDestroy(e);
        if (sv->flags) cudaFreeHost(sv->flags);
        pbf_batch_destroy(sv->batch);
    }
    delete sv;
    return PBF_OK;
}

}  // extern "C"

namespace {

struct CoupledArgs {
    int nb = 0;
    const float* local3 = nullptr;
    const int* body = nullptr;
    const float* psi = nullptr;
    int nbodies = 0;
    const pbf_rigid_body* bodies = nullptr;
    int nshapes = 0;
    const pbf_rigid_shape* shapes = nullptr;
    const pbf_contact_settings* cset = nullptr;
};

int open_impl(pbf_server* sv, const pbf_settings* st, int n, const float* x3, const float* v3,
              float mass, const float* g3, const CoupledArgs* cp, long long* id_out,
              int* state_out) {
    int rc = check_server(sv);
    if (rc) return rc;
    if (!st || !id_out || (n > 0 && !x3)) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    if (n < 0) return fail(PBF_ERR_INVALID_ARG, "n must be >= 0");
    rc = check_settings(st);
    if (rc) return rc;
    if (st->boundary_two_way)
        return fail(PBF_ERR_INVALID_ARG,
                    "boundary_two_way is not served: served coupled scenes use the reference's "
                    "one-way coupling");
    const uint32_t slots = grid_slots_for(*st, x3, n);
    size_t charge = charge_of(n, slots);
    if (cp) {
        if (cp->nb < 0 || cp->nbodies < 0 || (cp->nb > 0 && (!cp->local3 || !cp->body || !cp->psi)) ||
            (cp->nbodies > 0 && !cp->bodies))
            return fail(PBF_ERR_INVALID_ARG, "bad boundary or bodies");
        for (int i = 0; i < cp->nb; ++i)
            if (cp->body[i] >= cp->nbodies)
                return fail(PBF_ERR_INVALID_ARG, "a boundary particle names a missing body");
        if (cp->nshapes < 0 || (cp->nshapes > 0 && !cp->shapes))
            return fail(PBF_ERR_INVALID_ARG, "bad contact shapes");
        if (cp->nshapes > 16 || (cp->nshapes > 0 && cp->nbodies > 16))
            return fail(PBF_ERR_INVALID_ARG, "rigid contacts take at most 16 shapes and 16 bodies");
        for (int k = 0; k < cp->nshapes; ++k) {
            const pbf_rigid_shape& sh = cp->shapes[k];
            const bool sphere = sh.type == PBF_SHAPE_SPHERE && sh.body >= -1 && sh.body < cp->nbodies;
            const bool plane = sh.type == PBF_SHAPE_PLANE && sh.body == -1;
            if (!sphere && !plane)
                return fail(PBF_ERR_INVALID_ARG,
                            "contact shapes are spheres on existing bodies and world planes");
        }
        if (cp->cset && cp->cset->velocity_iterations < 0)
            return fail(PBF_ERR_INVALID_ARG, "velocity_iterations must be >= 0");
        // The coupling runs on the scene's own step scratch and offsets.
        charge += work_bytes(n > 0 ? n : 1) + sort_scratch_bytes(n > 0 ? n : 1) +
                  (size_t)slots * kGridBytesPerSlot + (size_t)cp->nb * kBoundaryBytes;
    }
    std::unique_lock<std::mutex> lk(sv->mu);
    if (charge + sv->scratch > sv->cfg.hbm_budget_bytes) {
        ++sv->rejected;
        return fail(PBF_ERR_CAPACITY, "the scene can never fit the HBM budget (" +
                                          std::to_string(charge) + " bytes charged)");
    }
    if (n > sv->cfg.max_batch_particles)
        return fail(PBF_ERR_CAPACITY, "the scene exceeds max_batch_particles");
    const long long id = sv->next_scene++;
    SceneRec& rec = sv->scenes[id];
    rec.id = id;
    rec.n = n;
    rec.charge = charge;
    rec.settings = *st;
    rec.mass = mass;
    if (g3)
        for (int d = 0; d < 3; ++d) rec.gravity[d] = g3[d];
    rec.x.assign(x3, x3 + (size_t)3 * n);
    if (v3) rec.v.assign(v3, v3 + (size_t)3 * n);
    if (cp) {
        rec.coupled = true;
        rec.local.assign(cp->local3, cp->local3 + (size_t)3 * cp->nb);
        rec.body.assign(cp->body, cp->body + cp->nb);
        rec.psi.assign(cp->psi, cp->psi + cp->nb);
        rec.bodies.assign(cp->bodies, cp->bodies + cp->nbodies);
        if (cp->nshapes > 0) rec.shapes.assign(cp->shapes, cp->shapes + cp->nshapes);
        if (cp->cset) rec.cset = *cp->cset;
    }
    sv->admit_queue.push_back(id);
    admit_waiting(sv, lk);
    auto it = sv->scenes.find(id);
    const int state = it == sv->scenes.end() ? PBF_SCENE_FAILED : it->second.state;
    *id_out = id;
    if (state_out) *state_out = state;
    return PBF_OK;
}

}  // namespace

extern "C" {

int pbf_server_open_scene(pbf_server* sv, const pbf_settings* st, int n, const float* x3,
                          const float* v3, float mass, const float* g3, long long* id_out,
                          int* state_out) {
    return open_impl(sv, st, n, x3, v3, mass, g3, nullptr, id_out, state_out);
}

int pbf_server_open_coupled_scene(pbf_server* sv, const pbf_settings* st, int n, const float* x3,
                                  const float* v3, float mass, const float* g3, int nb,
                                  const float* local3, const int* body, const float* psi,
                                  int nbodies, const pbf_rigid_body* bodies, long long* id_out,
                                  int* state_out) {
    CoupledArgs cp;
    cp.nb = nb;
    cp.local3 = local3;
    cp.body = body;
    cp.psi = psi;
    cp.nbodies = nbodies;
    cp.bodies = bodies;
    return open_impl(sv, st, n, x3, v3, mass, g3, &cp, id_out, state_out);
}

int pbf_server_open_coupled_scene_contacts(
    pbf_server* sv, const pbf_settings* st, int n, const float* x3, const float* v3, float mass,
    const float* g3, int nb, const float* local3, const int* body, const float* psi, int nbodies,
    const pbf_rigid_body* bodies, int nshapes, const pbf_rigid_shape* shapes,
    const pbf_contact_settings* cset, long long* id_out, int* state_out) {
    CoupledArgs cp;
    cp.nb = nb;
    cp.local3 = local3;
    cp.body = body;
    cp.psi = psi;
    cp.nbodies = nbodies;
    cp.bodies = bodies;
    cp.nshapes = nshapes;
    cp.shapes = shapes;
    cp.cset = cset;
    return open_impl(sv, st, n, x3, v3, mass, g3, &cp, id_out, state_out);
}

int pbf_server_close_scene(pbf_server* sv, long long id) {
    int rc = check_server(sv);
    if (rc) return rc;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->scenes.find(id);
    if (it == sv->scenes.end()) return fail(PBF_ERR_INVALID_ARG, "no such scene");
    // Let queued requests finish (a waiting scene has none running).
    sv->cv_done.wait(lk, [&] {
        auto i2 = sv->scenes.find(id);
        if (i2 == sv->scenes.end()) return true;
        const SceneRec& sc = i2->second;
        if (sc.busy) return false;
        if (sc.state == PBF_SCENE_WAITING) return true;
        for (long long rid : sc.reqs)
            if (req_pending(sv, rid)) return false;
        return sc.inflight == 0;
    });
    it = sv->scenes.find(id);
    if (it == sv->scenes.end()) return PBF_OK;
    SceneRec rec = std::move(it->second);
    sv->scenes.erase(it);
    for (long long rid : rec.reqs)
        if (ReqRec* r = find_req(sv, rid)) fail_request(sv, *r, "its scene was closed", PBF_ERR_INVALID_ARG);
    if (rec.state == PBF_SCENE_WAITING) {
        sv->admit_queue.erase(std::remove(sv->admit_queue.begin(), sv->admit_queue.end(), id),
                              sv->admit_queue.end());
    } else {
        sv->charged -= rec.charge;
    }
    lk.unlock();
    if (rec.s) pbf_scene_destroy(rec.s);
    lk.lock();
    admit_waiting(sv, lk);
    sv->cv_done.notify_all();
    return PBF_OK;
}

int pbf_server_submit(pbf_server* sv, long long scene, float dt, int nsteps, long long* req_out) {
    int rc = check_server(sv);
    if (rc) return rc;
    if (!req_out) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    if (!(dt > 0.0f) || !std::isfinite(dt)) return fail(PBF_ERR_INVALID_ARG, "dt must be > 0");
    if (nsteps < 0) return fail(PBF_ERR_INVALID_ARG, "nsteps must be >= 0");
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->scenes.find(scene);
    if (it == sv->scenes.end()) return fail(PBF_ERR_INVALID_ARG, "no such scene");
    SceneRec& sc = it->second;
    if (sc.state == PBF_SCENE_FAILED) return fail(sc.code, "the scene failed: " + sc.why);
    const double t = now_ms();
    const long long id = sv->next_req++;
    ReqRec& r = sv->reqs[id];
    r.id = id;
    r.scene = scene;
    r.dt = dt;
    r.nsteps = nsteps;
    r.t_submit = r.t_prev = t;
    ++sv->submitted;
    if (sv->t_first < 0.0) sv->t_first = t;
    *req_out = id;
    if (nsteps == 0 || sc.n == 0) {  // nothing to run (pbf_solver.cpp:21)
        r.state = PBF_REQ_DONE;
        ++sv->done_reqs;
        sv->req_ms.add(0.0);
        note_finished(sv, id);
        sv->cv_done.notify_all();
    } else {
        sc.reqs.push_back(id);
        sv->cv_work.notify_one();
    }
    return PBF_OK;
}

int pbf_server_wait(pbf_server* sv, long long rid, double timeout_s, int* state_out) {
    int rc = check_server(sv);
    if (rc) return rc;
    std::unique_lock<std::mutex> lk(sv->mu);
    const char* gone = "no such request (records of all but the latest 65536 finished requests are dropped)";
    if (!find_req(sv, rid)) return fail(PBF_ERR_INVALID_ARG, gone);
    auto done = [&] { return !req_pending(sv, rid); };
    if (timeout_s < 0.0) {
        sv->cv_done.wait(lk, done);
    } else if (!sv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) {
        if (state_out) *state_out = PBF_REQ_PENDING;
        return fail(PBF_ERR_TIMEOUT, "the request is still pending");
    }
    const ReqRec* r = find_req(sv, rid);
    if (!r) return fail(PBF_ERR_INVALID_ARG, gone);
    if (state_out) *state_out = r->state;
    if (r->state == PBF_REQ_FAILED) return fail(r->code, "the request failed: " + r->why);
    return PBF_OK;
}

int pbf_server_read(pbf_server* sv, long long id, int field, float* out) {
    int rc = check_server(sv);
    if (rc) return rc;
    if (!out) return fail(PBF_ERR_INVALID_ARG, "output is NULL");
    pbf_scene* s = nullptr;
    {
        std::unique_lock<std::mutex> lk(sv->mu);
        auto idle = [&] {
            auto i2 = sv->scenes.find(id);
            if (i2 == sv->scenes.end()) return true;
            const SceneRec& sc = i2->second;
            if (sc.busy) return false;
            for (long long r : sc.reqs)
                if (req_pending(sv, r)) return false;
            return sc.inflight == 0;
        };
        sv->cv_done.wait(lk, idle);
        auto it = sv->scenes.find(id);
        if (it == sv->scenes.end()) return fail(PBF_ERR_INVALID_ARG, "no such scene");
        if (it->second.state == PBF_SCENE_WAITING) {
            // Not on the device yet: the state is the host copy.
            const SceneRec& sc = it->second;
            const size_t n = (size_t)sc.n;
            if (field == PBF_FIELD_POSITIONS) {
                std::memcpy(out, sc.x.data(), n * 12);
            } else if (field == PBF_FIELD_VELOCITIES) {
                if (sc.v.empty()) std::memset(out, 0, n * 12);
                else std::memcpy(out, sc.v.data(), n * 12);
            } else if (field == PBF_FIELD_DENSITIES || field == PBF_FIELD_LAMBDAS) {
                std::memset(out, 0, n * 4);
            } else {
                return fail(PBF_ERR_INVALID_ARG, "unknown field");
            }
            return PBF_OK;
        }
        s = it->second.s;
        // No launch of this scene is pending; the busy flag keeps new launches
        // and close_scene away until the read is done.
        it->second.busy = true;
    }
    rc = s ? pbf_scene_read(s, field, out) : fail(PBF_ERR_INVALID_ARG, "scene has no device copy");
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        auto it = sv->scenes.find(id);
        if (it != sv->scenes.end()) it->second.busy = false;
    }
    sv->cv_done.notify_all();
    return rc;
}

int pbf_server_read_bodies(pbf_server* sv, long long id, pbf_rigid_body* out) {
    int rc = check_server(sv);
    if (rc) return rc;
    pbf_scene* s = nullptr;
    {
        std::unique_lock<std::mutex> lk(sv->mu);
        sv->cv_done.wait(lk, [&] {
            auto it = sv->scenes.find(id);
            if (it == sv->scenes.end()) return true;
            const SceneRec& sc = it->second;
            if (sc.busy || sc.inflight > 0) return false;
            for (long long r : sc.reqs)
                if (req_pending(sv, r)) return false;
            return true;
        });
        auto it = sv->scenes.find(id);
        if (it == sv->scenes.end()) return fail(PBF_ERR_INVALID_ARG, "no such scene");
        SceneRec& sc = it->second;
        const auto& b = sc.bodies;
        if (!b.empty() && !out) return fail(PBF_ERR_INVALID_ARG, "output is NULL");
        if (!sc.s || b.empty()) {  // not on the device yet: the host copy
            std::copy(b.begin(), b.end(), out);
            return PBF_OK;
        }
        // The bodies step on the device, after the scene's last step; the busy
        // flag keeps launches and close_scene away while they are copied.
        s = sc.s;
        sc.busy = true;
    }
    rc = scene_read_rigid(s, out);
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        auto it = sv->scenes.find(id);
        if (it != sv->scenes.end()) it->second.busy = false;
    }
    sv->cv_done.notify_all();
    return rc;
}

int pbf_server_scene_state(pbf_server* sv, long long id, int* state_out) {
    int rc = check_server(sv);
    if (rc) return rc;
    if (!state_out) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->scenes.find(id);
    if (it == sv->scenes.end()) return fail(PBF_ERR_INVALID_ARG, "no such scene");
    *state_out = it->second.state;
    return PBF_OK;
}

int pbf_server_get_stats(pbf_server* sv, pbf_server_stats* out) {
    int rc = check_server(sv);
    if (rc) return rc;
    if (!out) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    pbf_server_stats s{};
    for (auto& kv : sv->scenes) {
        if (kv.second.state == PBF_SCENE_WAITING) ++s.scenes_waiting;
        else if (kv.second.state == PBF_SCENE_RESIDENT) ++s.scenes_resident;
    }
    s.scenes_rejected = sv->rejected;
    s.scenes_failed = sv->failed_scenes;
    s.requests_submitted = sv->submitted;
    s.requests_done = sv->done_reqs;
    s.requests_failed = sv->failed_reqs;
    s.steps_done = sv->steps_done;
    s.particle_steps = sv->particle_steps;
    s.launches = sv->launches;
    s.queue_depth = sv->submitted - sv->done_reqs - sv->failed_reqs;
    s.step_ms_p50 = sv->step_ms.percentile(50.0);
    s.step_ms_p99 = sv->step_ms.percentile(99.0);
    s.request_ms_p50 = sv->req_ms.percentile(50.0);
    s.request_ms_p99 = sv->req_ms.percentile(99.0);
    const double span = sv->t_last - sv->t_first;
    s.particle_steps_per_s = (sv->t_first >= 0.0 && span > 0.0)
                                 ? (double)sv->particle_steps / (span / 1e3)
                                 : 0.0;
    s.mean_launch_scenes = sv->launches ? (double)sv->launch_scenes / sv->launches : 0.0;
    s.mean_launch_particles = sv->launches ? (double)sv->launch_particles / sv->launches : 0.0;
    s.hbm_bytes_charged = sv->charged;
    s.hbm_bytes_scratch = sv->scratch;
    s.state_bytes_per_particle = kStateBytesPerParticle;
    s.grid_bytes_per_slot = kGridBytesPerSlot;
    s.issue_ms_mean = sv->launches ? sv->issue_ms / sv->launches : 0.0;
    s.post_ms_mean = sv->launches ? sv->post_ms / sv->launches : 0.0;
    batch_counters(sv->batch, &s.graph_captures, &s.graph_updates, &s.graph_instantiations,
                   &s.launches_direct);
    *out = s;
    return PBF_OK;
}

int pbf_server_reset_stats(pbf_server* sv) {
    int rc = check_server(sv);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->submitted -= sv->done_reqs + sv->failed_reqs;
    sv->done_reqs = sv->failed_reqs = 0;
    sv->steps_done = sv->particle_steps = sv->launches = 0;
    sv->launch_scenes = sv->launch_particles = 0;
    sv->issue_ms = 0.0;
    sv->post_ms = 0.0;
    sv->rejected = 0;
    sv->t_first = -1.0;
    sv->t_last = 0.0;
    sv->step_ms.clear();
    sv->req_ms.clear();
    for (auto it = sv->reqs.begin(); it != sv->reqs.end();) {
        if (it->second.state != PBF_REQ_PENDING) it = sv->reqs.erase(it);
        else ++it;
    }
    sv->finished.clear();
    return PBF_OK;
}

}  // extern "C"
