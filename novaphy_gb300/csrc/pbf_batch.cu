// C ABI of batched stepping (include/novaphy_pbf.h, "Batches of scenes"):
// many independent scenes share one cell-key sort, one reference-key sort and
// one kernel launch per phase.  Each scene keeps its state in place; the
// kernels reach it through a per-scene table (state pointers, particle range,
// step constants, slot range) uploaded before every step.
//
// The batch's particle order is the concatenation of the scenes' particle
// orders and its cell-slot space the concatenation of their grids, so within
// a scene every sort is stable in the scene's own particle order and every
// neighbour walk visits the same candidates in the same order as a step of
// the scene alone: results do not depend on what else is in the batch.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "pbf_internal.cuh"
#include "pbf_launch.cuh"

using namespace pbf;
using namespace pbf::capi;

namespace {

// The launch sequence of a batch step depends on these; a cached graph is
// reused (with updated kernel parameters) while they stay the same.
struct GraphKey {
    int exact = -1, persist = 0, block = 0, n = 0, nscenes = 0, key_bits = 0, scene_bits = 0,
        max_iters = 0;
    uint32_t nslots = 0;
    bool any_zero = false, any_vort = false, any_plain = false, xsph_on = false;
    bool operator==(const GraphKey& o) const {
        return exact == o.exact && persist == o.persist && block == o.block && n == o.n &&
               nscenes == o.nscenes &&
               key_bits == o.key_bits &&
               scene_bits == o.scene_bits && max_iters == o.max_iters && nslots == o.nslots &&
               any_zero == o.any_zero && any_vort == o.any_vort && any_plain == o.any_plain &&
               xsph_on == o.xsph_on;
    }
};

int bits_for(unsigned long long v) {
    int b = 1;
    while ((1ull << b) < v) ++b;
    return b;
}

// Autotuning.  A choice is the block size of the neighbour passes and
// whether the Jacobi loop runs as one persistent launch.  A class of batch
// shapes tries each choice once, on its next steps, and keeps the fastest.
struct Choice {
    int block = 128;
    int persist = 0;
};

const Choice kChoices[] = {{128, 0}, {64, 0}, {256, 0}, {128, 1}};
constexpr int kNumChoices = (int)(sizeof(kChoices) / sizeof(kChoices[0]));

struct TuneState {
    bool done = false;
    Choice best;
    double best_ms = 0.0;
    int next = 0;              // next choice to try
    int pending = -1;          // choice whose timing is in flight
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    // A trial whose step failed before its timing was recorded keeps +inf
    // and is never chosen.
    double ms[kNumChoices];
    TuneState() {
        for (double& m : ms) m = 1e30;
    }
};

}  // namespace

struct pbf_batch {
    int device = 0;
    // Private to the batch: only calls holding `mu` enqueue work on it, so a
    // graph capture on it records the step's work and nothing else.
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    std::mutex mu;

    int cap = 0;  // particles
    void* wmem = nullptr;  // step scratch (bind_work)
    void* smem = nullptr;  // sort scratch
    void* xmem = nullptr;  // scene ids, scene-pass temporaries
    StepBuffers B{};
    SortScratch sort{};
    uint32_t *pid = nullptr, *spid = nullptr, *kpid = nullptr, *itmp = nullptr, *perm = nullptr,
             *stmp = nullptr;
    unsigned long long* rtmp = nullptr;

    uint32_t* off = nullptr;  // nslots + 1 offsets, then one alias byte per slot
    uint32_t off_cap = 0;     // entries

    int tab_cap = 0;  // scenes
    void* tmem = nullptr;  // per-scene tables: StepConsts | StateRef | firsts
    size_t tab_refs_at = 0, tab_firsts_at = 0, tab_bytes = 0;
    // Pinned host copies of the tables, used in turn and allocated on first
    // use; each one's event marks the end of its upload, so it is rewritten
    // only after the copy is done.  Sized for the step uploads that can be
    // queued at once (a serving launch runs up to 16 steps, two launches in
    // flight), so that issuing a step does not wait for the device.
    static constexpr int kTabRing = 64;
    char* h_tab[kTabRing] = {};
    cudaEvent_t h_tab_ev[kTabRing] = {};
    bool h_tab_used[kTabRing] = {};
    int h_tab_next = 0;

    cudaEvent_t fork = nullptr;  // splits scenes' post-steps off between steps
    uint32_t* d_bad = nullptr;  // per-scene non-finite flags of the last call
    int bad_cap = 0;
    int bad_count = 0;

    // Persistent Jacobi loop (one cooperative launch per step) when set.
    bool persistent = false;
    int persist_blocks[2] = {-1, -1};  // co-resident grid per build (fast, exact)
    unsigned int* barrier = nullptr;   // grid barrier words

    // One cached step graph per arithmetic build (index: exact), so a call
    // that steps scenes of both builds does not recapture every group.
    cudaGraphExec_t graph[2] = {};
    GraphKey key[2];
    // A shape is captured the second time in a row it is seen; a shape seen
    // once (a serving loop's launches change shape nearly every time) is
    // launched directly, which costs far less host time than a capture.
    GraphKey seen[2];
    long long direct = 0;
    long long captures = 0, updates = 0, instantiations = 0;

    // Autotuner (off by default): per class of batch shape.
    bool autotune = false;
    std::string gpu;
    std::string cache_path;
    std::map<std::string, TuneState> tune;
    Choice last{};
};

namespace {

void drop_graph(pbf_batch* b) {
    for (int k = 0; k < 2; ++k) {
        if (b->graph[k]) cudaGraphExecDestroy(b->graph[k]);
        b->graph[k] = nullptr;
        b->key[k] = GraphKey{};
    }
}

size_t extra_bytes(int c) {
    return 6 * align_up((size_t)c * 4, 256) + align_up((size_t)c * 8, 256);
}

int ensure_particles(pbf_batch* b, int n) {
    if (b->wmem && b->cap >= n) return PBF_OK;
    drop_graph(b);
    for (void* m : {b->wmem, b->smem, b->xmem})
        if (m) cudaFree(m);
    b->wmem = b->smem = b->xmem = nullptr;
    b->cap = 0;
    // Grow by a quarter so that a slowly growing batch does not reallocate
    // on every step.
    const int c = std::max(n + n / 4, 1024);
    const size_t wb = work_bytes(c);
    PBF_CUDA(cudaMalloc(&b->wmem, wb));
    PBF_CUDA(cudaMemsetAsync(b->wmem, 0, wb, b->stream));
    bind_work(b->B, b->wmem, c);
    const size_t sb = sort_scratch_bytes(c);
    PBF_CUDA(cudaMalloc(&b->smem, sb));
    PBF_CUDA(cudaMemsetAsync(b->smem, 0, sb, b->stream));
    sort_scratch_bind(b->sort, b->smem, c);
    b->B.err = b->sort.err;
    const size_t xb = extra_bytes(c);
    PBF_CUDA(cudaMalloc(&b->xmem, xb));
    char* p = reinterpret_cast<char*>(b->xmem);
    const size_t f1 = align_up((size_t)c * 4, 256);
    uint32_t** arr[6] = {&b->pid, &b->spid, &b->kpid, &b->itmp, &b->perm, &b->stmp};
    for (int k = 0; k < 6; ++k) *arr[k] = reinterpret_cast<uint32_t*>(p + k * f1);
    b->rtmp = reinterpret_cast<unsigned long long*>(p + 6 * f1);
    b->cap = c;
    return PBF_OK;
}

int ensure_slots(pbf_batch* b, uint32_t nslots) {
    if (b->off && b->off_cap >= nslots + 1) return PBF_OK;
    drop_graph(b);
    if (b->off) cudaFree(b->off);
    b->off = nullptr;
    b->off_cap = 0;
    const uint32_t c = nslots + nslots / 4 + 1;
    const size_t ob = align_up((size_t)(c + 1) * 4, 256);
    const size_t ab = align_up(c + 1, 256);
    PBF_CUDA(cudaMalloc(&b->off, ob + ab + (size_t)(c + 1) * 8));
    b->off_cap = c + 1;
    b->B.off = b->off;
    b->B.slot_alias = reinterpret_cast<unsigned char*>(b->off) + ob;
    b->B.moved = reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(b->off) + ob + ab);
    b->B.lamnz = b->B.moved + (c + 1);
    return PBF_OK;
}

void free_tables(pbf_batch* b) {
    if (b->tmem) cudaFree(b->tmem);
    b->tmem = nullptr;
    for (int k = 0; k < pbf_batch::kTabRing; ++k) {
        if (b->h_tab_ev[k]) {
            cudaEventSynchronize(b->h_tab_ev[k]);
            cudaEventDestroy(b->h_tab_ev[k]);
        }
        if (b->h_tab[k]) cudaFreeHost(b->h_tab[k]);
        b->h_tab[k] = nullptr;
        b->h_tab_ev[k] = nullptr;
        b->h_tab_used[k] = false;
    }
    b->tab_cap = 0;
}

int ensure_tables(pbf_batch* b, int nscenes) {
    if (b->tmem && b->tab_cap >= nscenes) return PBF_OK;
    drop_graph(b);
    free_tables(b);
    const int c = std::max(nscenes + nscenes / 4, 64);
    b->tab_refs_at = align_up((size_t)c * sizeof(StepConsts), 256);
    b->tab_firsts_at = b->tab_refs_at + align_up((size_t)c * sizeof(StateRef), 256);
    b->tab_bytes = b->tab_firsts_at + align_up((size_t)(c + 1) * 4, 256);
    PBF_CUDA(cudaMalloc(&b->tmem, b->tab_bytes));
    b->tab_cap = c;
    return PBF_OK;
}

int ensure_bad(pbf_batch* b, int nscenes) {
    if (b->d_bad && b->bad_cap >= nscenes) return PBF_OK;
    drop_graph(b);
    if (b->d_bad) cudaFree(b->d_bad);
    b->d_bad = nullptr;
    b->bad_cap = 0;
    const int c = std::max(nscenes + nscenes / 4, 64);
    PBF_CUDA(cudaMalloc(&b->d_bad, (size_t)c * 4));
    b->bad_cap = c;
    return PBF_OK;
}

bool graphs_enabled() {
    const char* v = std::getenv("PBF_NO_GRAPH");
    return !(v && v[0] == '1');
}

// Where tuning decisions are kept: $PBF_AUTOTUNE_CACHE, else
// ~/.cache/novaphy_gb300/autotune.jsonl.  One JSON object per line.
std::string cache_file() {
    if (const char* p = std::getenv("PBF_AUTOTUNE_CACHE")) return p;
    const char* home = std::getenv("HOME");
    return std::string(home ? home : ".") + "/.cache/novaphy_gb300/autotune.jsonl";
}

// Value of "key": in one of our own cache lines (string or number).
std::string json_field(const std::string& line, const std::string& key) {
    const std::string k = "\"" + key + "\": ";
    const size_t at = line.find(k);
    if (at == std::string::npos) return {};
    size_t b = at + k.size();
    if (b < line.size() && line[b] == '"') {
        const size_t e = line.find('"', b + 1);
        return e == std::string::npos ? std::string() : line.substr(b + 1, e - b - 1);
    }
    size_t e = line.find_first_of(",}", b);
    return line.substr(b, e == std::string::npos ? std::string::npos : e - b);
}

void load_tuning(pbf_batch* b) {
    std::ifstream in(b->cache_path);
    std::string line;
    while (std::getline(in, line)) {
        if (json_field(line, "gpu") != b->gpu) continue;
        const std::string cls = json_field(line, "class");
        const std::string block = json_field(line, "block"), persist = json_field(line, "persistent");
        if (cls.empty() || block.empty() || persist.empty()) continue;
        TuneState& t = b->tune[cls];
        t.done = true;
        t.best.block = std::atoi(block.c_str());
        t.best.persist = std::atoi(persist.c_str());
        t.best_ms = std::atof(json_field(line, "ms").c_str());
    }
}

void save_tuning(const pbf_batch* b, const std::string& cls, const TuneState& t) {
    const std::string& path = b->cache_path;
    const size_t slash = path.find_last_of('/');
    if (slash != std::string::npos) {
        // mkdir -p of the cache directory, one level at a time
        for (size_t at = path.find('/', 1); at != std::string::npos && at <= slash;
             at = path.find('/', at + 1))
            (void)mkdir(path.substr(0, at).c_str(), 0755);
    }
    std::ofstream out(path, std::ios::app);
    if (!out) return;  // a cache that cannot be written only costs re-tuning
    out << "{\"gpu\": \"" << b->gpu << "\", \"class\": \"" << cls << "\", \"block\": "
        << t.best.block << ", \"persistent\": " << t.best.persist << ", \"ms\": " << t.best_ms
        << "}\n";
}

// Class of a batch shape: arithmetic build, particle-count octave, largest
// iteration count, vorticity on any scene.
std::string tune_class(int exact, int n, int max_iters, bool any_vort) {
    std::ostringstream o;
    o << (exact ? "exact" : "fast") << " n2^" << bits_for((unsigned long long)n) << " it"
      << max_iters << (any_vort ? " vort" : "");
    return o.str();
}

// The choice for this step of class `cls`; collects the timing of the
// previous trial first.
Choice pick_choice(pbf_batch* b, const std::string& cls, int* trial) {
    *trial = -1;
    TuneState& t = b->tune[cls];
    if (t.pending >= 0) {
        float ms = 0.0f;
        if (cudaEventSynchronize(t.e1) == cudaSuccess &&
            cudaEventElapsedTime(&ms, t.e0, t.e1) == cudaSuccess)
            t.ms[t.pending] = ms;
        else
            t.ms[t.pending] = 1e30;
        t.pending = -1;
    }
    if (!t.done && t.next >= kNumChoices) {
        // Every choice was tried (a trial whose step failed kept +inf).
        int best = 0;
        for (int k = 1; k < kNumChoices; ++k)
            if (t.ms[k] < t.ms[best]) best = k;
        t.done = true;
        if (t.ms[best] < 1e30) {
            t.best = kChoices[best];
            t.best_ms = t.ms[best];
            save_tuning(b, cls, t);
        }
    }
    if (t.done) return t.best;
    if (!t.e0 && (cudaEventCreate(&t.e0) != cudaSuccess || cudaEventCreate(&t.e1) != cudaSuccess)) {
        // No timing events: keep the default choice and stop tuning this class.
        cudaGetLastError();
        t.done = true;
        return t.best;
    }
    *trial = t.next++;
    return kChoices[*trial];
}

// One step of `list` (scenes with particles, all of one arithmetic build):
// per-scene tables uploaded, then the batch's launch sequence (from a graph).
int step_group(pbf_batch* b, const std::vector<pbf_scene*>& list, const std::vector<float>& dts,
               const std::vector<int>& orig, int exact, PhaseMarks* pm) {
    const int ns = (int)list.size();
    if (ns == 0) return PBF_OK;
    unsigned long long n_total = 0, slots_total = 0;
    int max_iters = 0;
    bool any_zero = false, any_vort = false, any_plain = false, xsph_on = false;
    std::vector<StepConsts> consts((size_t)ns);
    for (int k = 0; k < ns; ++k) {
        pbf_scene* s = list[k];
        StepConsts& C = consts[k];
        int rc = scene_consts(s, dts[k], C);
        if (rc) return rc;
        C.seg_begin = (uint32_t)n_total;
        C.seg_end = (uint32_t)(n_total + (unsigned long long)s->n);
        C.grid.base = (uint32_t)slots_total;
        n_total += (unsigned long long)s->n;
        slots_total += C.grid.nslots;
        if (n_total > (1ull << 30)) return fail(PBF_ERR_CAPACITY, "at most 2^30 particles per batch");
        if (slots_total > (1ull << 30))
            return fail(PBF_ERR_CAPACITY, "the scenes' grids exceed 2^30 cell slots in total");
        max_iters = std::max(max_iters, C.iters);
        any_zero |= C.iters <= 0;
        any_vort |= C.vort_on != 0;
        any_plain |= C.vort_on == 0;
        xsph_on |= C.xsph_on != 0;
    }
    const int n = (int)n_total;
    int rc = ensure_particles(b, n);
    if (!rc) rc = ensure_slots(b, (uint32_t)slots_total);
    if (!rc) rc = ensure_tables(b, ns);
    if (rc) return rc;

    const int ring = b->h_tab_next;
    b->h_tab_next = (ring + 1) % pbf_batch::kTabRing;
    if (!b->h_tab[ring]) {
        PBF_CUDA(cudaMallocHost(&b->h_tab[ring], b->tab_bytes));
        PBF_CUDA(cudaEventCreateWithFlags(&b->h_tab_ev[ring], cudaEventDisableTiming));
    }
    if (b->h_tab_used[ring]) PBF_CUDA(cudaEventSynchronize(b->h_tab_ev[ring]));
    char* h = b->h_tab[ring];
    auto* htab = reinterpret_cast<StepConsts*>(h);
    auto* hrefs = reinterpret_cast<StateRef*>(h + b->tab_refs_at);
    auto* hfirst = reinterpret_cast<uint32_t*>(h + b->tab_firsts_at);
    for (int k = 0; k < ns; ++k) {
        pbf_scene* s = list[k];
        htab[k] = consts[k];
        hrefs[k] = StateRef{s->B.x, s->B.v, s->B.rho, s->B.lam, consts[k].seg_begin,
                            b->d_bad + orig[k]};
        hfirst[k] = consts[k].seg_begin;
    }
    hfirst[ns] = (uint32_t)n;
    PBF_CUDA(cudaMemcpyAsync(b->tmem, h, b->tab_firsts_at + (size_t)(ns + 1) * 4,
                             cudaMemcpyHostToDevice, b->stream));
    PBF_CUDA(cudaEventRecord(b->h_tab_ev[ring], b->stream));
    b->h_tab_used[ring] = true;

    BatchDesc D{};
    D.n = n;
    D.nscenes = ns;
    D.nslots = (uint32_t)slots_total;
    D.key_bits = bits_for(slots_total);
    D.scene_bits = bits_for((unsigned long long)ns);
    D.max_iters = max_iters;
    D.any_zero_iters = any_zero;
    D.any_vort = any_vort;
    D.any_plain = any_plain;
    D.xsph_on = xsph_on;
    char* t = reinterpret_cast<char*>(b->tmem);
    D.tab = reinterpret_cast<const StepConsts*>(t);
    D.refs = reinterpret_cast<const StateRef*>(t + b->tab_refs_at);
    D.firsts = reinterpret_cast<const uint32_t*>(t + b->tab_firsts_at);
    D.pid = b->pid;
    D.spid = b->spid;
    D.kpid = b->kpid;
    D.rtmp = b->rtmp;
    D.itmp = b->itmp;
    D.perm = b->perm;
    D.stmp = b->stmp;
    D.persist_blocks = 0;
    D.barrier = b->barrier;
    Choice choice;
    choice.persist = b->persistent ? 1 : 0;
    int trial = -1;
    std::string cls;
    if (b->autotune && !pm) {
        cls = tune_class(exact, n, max_iters, any_vort);
        choice = pick_choice(b, cls, &trial);
    }
    D.block = choice.block;
    if (choice.persist && max_iters > 0) {
        int& pb = b->persist_blocks[exact];
        if (pb < 0) pb = exact ? exact_persist_blocks() : fast_persist_blocks();
        D.persist_blocks = pb;
    }
    b->last = choice;
    TuneState* ts = trial >= 0 ? &b->tune[cls] : nullptr;

    auto enqueue = [&](cudaStream_t st, PhaseMarks* marks) {
        return exact ? exact_enqueue_batch(b->B, D, b->sort, st, marks)
                     : fast_enqueue_batch(b->B, D, b->sort, st, marks);
    };
    if (pm || !graphs_enabled()) {
        if (ts) PBF_CUDA(cudaEventRecord(ts->e0, b->stream));
        cudaError_t e = enqueue(b->stream, pm);
        if (e != cudaSuccess) return cuda_fail(e, "batch step");
        if (ts) {
            PBF_CUDA(cudaEventRecord(ts->e1, b->stream));
            ts->pending = trial;
        }
        return PBF_OK;
    }
    GraphKey key;
    key.exact = exact;
    key.persist = D.persist_blocks;
    key.block = D.block;
    key.n = n;
    key.nscenes = ns;
    key.key_bits = D.key_bits;
    key.scene_bits = D.scene_bits;
    key.max_iters = max_iters;
    key.nslots = D.nslots;
    key.any_zero = any_zero;
    key.any_vort = any_vort;
    key.any_plain = any_plain;
    key.xsph_on = xsph_on;
    cudaGraphExec_t& graph = b->graph[exact];
    const bool cached = graph && key == b->key[exact];
    if (!cached && !(key == b->seen[exact])) {
        b->seen[exact] = key;
        ++b->direct;
        if (ts) PBF_CUDA(cudaEventRecord(ts->e0, b->stream));
        cudaError_t e = enqueue(b->stream, nullptr);
        if (e != cudaSuccess) return cuda_fail(e, "batch step");
        if (ts) {
            PBF_CUDA(cudaEventRecord(ts->e1, b->stream));
            ts->pending = trial;
        }
        return PBF_OK;
    }
    if (!cached) {
        ++b->captures;
        cudaGraph_t g = nullptr;
        PBF_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        const cudaError_t ee = enqueue(b->stream, nullptr);
        cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
        if (ee != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return cuda_fail(ee, "batch step (capture)");
        }
        if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
        bool updated = false;
        if (graph) {
            // Same launch topology with new sizes: update the parameters in place.
            cudaGraphExecUpdateResultInfo info{};
            updated = cudaGraphExecUpdate(graph, g, &info) == cudaSuccess;
            if (updated) ++b->updates;
            if (!updated) {
                cudaGetLastError();
                cudaGraphExecDestroy(graph);
                graph = nullptr;
            }
        }
        if (!updated) {
            ++b->instantiations;
            ce = cudaGraphInstantiate(&graph, g, 0);
            if (ce != cudaSuccess) {
                cudaGraphDestroy(g);
                graph = nullptr;
                return cuda_fail(ce, "cudaGraphInstantiate");
            }
        }
        cudaGraphDestroy(g);
        b->key[exact] = key;
    }
    if (ts) PBF_CUDA(cudaEventRecord(ts->e0, b->stream));
    PBF_CUDA(cudaGraphLaunch(graph, b->stream));
    if (ts) {
        PBF_CUDA(cudaEventRecord(ts->e1, b->stream));
        ts->pending = trial;
    }
    return PBF_OK;
}

// Locks the scenes (in address order, so that concurrent batches over
// overlapping sets cannot deadlock) and checks them.
struct SceneLocks {
    std::vector<std::unique_lock<std::mutex>> locks;
};

int lock_scenes(const pbf_batch* b, int nscenes, pbf_scene* const* scenes, SceneLocks& L) {
    std::vector<pbf_scene*> sorted(scenes, scenes + nscenes);
    for (pbf_scene* s : sorted)
        if (!s) return fail(PBF_ERR_INVALID_ARG, "a scene is NULL");
    std::sort(sorted.begin(), sorted.end());
    if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
        return fail(PBF_ERR_INVALID_ARG, "a scene appears twice in the batch");
    for (pbf_scene* s : sorted)
        if (s->device != b->device) return fail(PBF_ERR_INVALID_ARG, "a scene is on another device");
    L.locks.reserve(sorted.size());
    for (pbf_scene* s : sorted) L.locks.emplace_back(s->mu);
    return PBF_OK;
}

// Orders the batch stream after each scene's stream.
int wait_for_scenes(pbf_batch* b, int nscenes, pbf_scene* const* scenes) {
    for (int k = 0; k < nscenes; ++k) {
        pbf_scene* s = scenes[k];
        if (!s->ev) PBF_CUDA(cudaEventCreateWithFlags(&s->ev, cudaEventDisableTiming));
        PBF_CUDA(cudaEventRecord(s->ev, s->stream));
        PBF_CUDA(cudaStreamWaitEvent(b->stream, s->ev, 0));
    }
    return PBF_OK;
}

// Orders each scene's later work after the batch.
int release_scenes(pbf_batch* b, int nscenes, pbf_scene* const* scenes) {
    PBF_CUDA(cudaEventRecord(b->done, b->stream));
    for (int k = 0; k < nscenes; ++k) PBF_CUDA(cudaStreamWaitEvent(scenes[k]->stream, b->done, 0));
    return PBF_OK;
}

int run_batch(pbf_batch* b, int nscenes, pbf_scene* const* scenes, const float* dt,
              const int* nsteps, const LaunchSpec* spec = nullptr) {
    int max_steps = 0;
    for (int k = 0; k < nscenes; ++k) {
        const int m = nsteps ? nsteps[k] : 1;
        if (m < 0) return fail(PBF_ERR_INVALID_ARG, "nsteps must be >= 0");
        if (!(dt[k] > 0.0f) || !std::isfinite(dt[k]))
            return fail(PBF_ERR_INVALID_ARG, "dt must be > 0");
        max_steps = std::max(max_steps, m);
    }
    int rc = ensure_bad(b, nscenes);
    if (rc) return rc;
    b->bad_count = nscenes;
    if (nscenes > 0) PBF_CUDA(cudaMemsetAsync(b->d_bad, 0, (size_t)nscenes * 4, b->stream));
    std::vector<pbf_scene*> list;
    std::vector<float> dts;
    std::vector<int> orig;
    list.reserve((size_t)nscenes);
    dts.reserve((size_t)nscenes);
    orig.reserve((size_t)nscenes);
    for (int step = 0; step < max_steps; ++step) {
        for (int exact = 1; exact >= 0; --exact) {
            list.clear();
            dts.clear();
            orig.clear();
            for (int k = 0; k < nscenes; ++k) {
                pbf_scene* s = scenes[k];
                const int m = nsteps ? nsteps[k] : 1;
                if (step >= m || s->n <= 0) continue;  // pbf_solver.cpp:21
                if ((s->settings.exact_arithmetic ? 1 : 0) != exact) continue;
                list.push_back(s);
                dts.push_back(dt[k]);
                orig.push_back(k);
            }
            rc = step_group(b, list, dts, orig, exact, nullptr);
            if (rc) return rc;
        }
        if (spec && spec->sub && step < spec->nsub)
            PBF_CUDA(cudaEventRecord(spec->sub[step], b->stream));
        if (spec && spec->post && step + 1 < max_steps) {
            // Post-steps of the scenes that step again, forked off the batch
            // stream onto their own streams and joined before the next step.
            bool forked = false;
            for (int k = 0; k < nscenes; ++k) {
                pbf_scene* s = scenes[k];
                const int m = nsteps ? nsteps[k] : 1;
                if (!spec->needs_post || !spec->needs_post[k] || m <= step + 1 || s->n <= 0)
                    continue;
                if (!forked) {
                    if (!b->fork)
                        PBF_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
                    PBF_CUDA(cudaEventRecord(b->fork, b->stream));
                    forked = true;
                }
                PBF_CUDA(cudaStreamWaitEvent(s->stream, b->fork, 0));
                rc = spec->post(spec->post_ctx, s, k);
                if (rc) return rc;
                if (!s->ev) PBF_CUDA(cudaEventCreateWithFlags(&s->ev, cudaEventDisableTiming));
                PBF_CUDA(cudaEventRecord(s->ev, s->stream));
                PBF_CUDA(cudaStreamWaitEvent(b->stream, s->ev, 0));
            }
        }
    }
    return PBF_OK;
}

int batch_sync(pbf_batch* b) {
    PBF_CUDA(cudaStreamSynchronize(b->stream));
    if (!b->sort.err) return PBF_OK;
    uint32_t err = 0;
    PBF_CUDA(cudaMemcpy(&err, b->sort.err, 4, cudaMemcpyDeviceToHost));
    if (err) {
        PBF_CUDA(cudaMemset(b->sort.err, 0, 4));
        return fail(PBF_ERR_TIMEOUT, "a device-side wait of a batch step gave up (error word " +
                                         std::to_string(err) + ")");
    }
    return PBF_OK;
}

int check_args(pbf_batch* b, int nscenes, pbf_scene* const* scenes, const float* dt) {
    if (!b) return fail(PBF_ERR_INVALID_ARG, "batch is NULL");
    if (nscenes < 0) return fail(PBF_ERR_INVALID_ARG, "nscenes must be >= 0");
    if (nscenes > 0 && (!scenes || !dt)) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    for (int k = 0; k < nscenes; ++k)
        if (scenes[k] && scenes[k]->settings.boundary_two_way && scenes[k]->bnd.nb > 0)
            return fail(PBF_ERR_INVALID_ARG,
                        "boundary_two_way steps run through pbf_scene_step_coupled; a batch "
                        "steps the fluid without its boundary");
    return PBF_OK;
}

}  // namespace

namespace pbf {
namespace capi {

int batch_launch(pbf_batch* b, const LaunchSpec& S) {
    std::lock_guard<std::mutex> lk(b->mu);
    DeviceGuard dg(b->device);
    SceneLocks L;
    const int nscenes = S.nscenes;
    int rc = lock_scenes(b, nscenes, S.scenes, L);
    if (rc) return rc;
    rc = wait_for_scenes(b, nscenes, S.scenes);
    if (!rc && S.start && cudaEventRecord(S.start, b->stream) != cudaSuccess)
        rc = fail(PBF_ERR_CUDA, "start event");
    if (!rc) rc = run_batch(b, nscenes, S.scenes, S.dt, S.nsteps, &S);
    if (!rc && S.flags_host && nscenes > 0)
        rc = cudaMemcpyAsync(S.flags_host, b->d_bad, (size_t)nscenes * 4, cudaMemcpyDeviceToHost,
                             b->stream) == cudaSuccess
                 ? PBF_OK
                 : fail(PBF_ERR_CUDA, "flags copy");
    const int rc2 = release_scenes(b, nscenes, S.scenes);
    if (!rc && S.done) PBF_CUDA(cudaEventRecord(S.done, b->stream));
    return rc ? rc : rc2;
}

void batch_counters(const pbf_batch* b, long long* captures, long long* updates,
                    long long* instantiations, long long* direct) {
    *direct = b->direct;
    *captures = b->captures;
    *updates = b->updates;
    *instantiations = b->instantiations;
}

int batch_reserve(pbf_batch* b, int particles, int scenes) {
    std::lock_guard<std::mutex> lk(b->mu);
    DeviceGuard dg(b->device);
    int rc = ensure_particles(b, particles);
    if (!rc) rc = ensure_tables(b, scenes);
    if (!rc) rc = ensure_bad(b, scenes);
    return rc;
}

size_t batch_bytes(const pbf_batch* b) {
    size_t t = 0;
    if (b->wmem) t += work_bytes(b->cap) + sort_scratch_bytes(b->cap) + extra_bytes(b->cap);
    if (b->off)
        t += align_up((size_t)b->off_cap * 4, 256) + align_up(b->off_cap, 256) +
             (size_t)b->off_cap * 8;
    t += b->tab_bytes + (size_t)b->bad_cap * 4;
    return t;
}

}  // namespace capi
}  // namespace pbf

extern "C" {

int pbf_batch_create(int device, pbf_batch** out) {
    if (!out) return fail(PBF_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    int count = 0;
    cudaError_t ce = cudaGetDeviceCount(&count);
    if (ce != cudaSuccess || count == 0)
        return fail(PBF_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(ce));
    if (device < 0 || device >= count) return fail(PBF_ERR_INVALID_ARG, "device out of range");
    DeviceGuard dg(device);
    if (!dg.ok) return fail(PBF_ERR_NO_DEVICE, "cudaSetDevice failed");
    std::unique_ptr<pbf_batch> b(new pbf_batch());
    b->device = device;
    PBF_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    ce = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaMalloc(&b->barrier, 256);
    if (ce == cudaSuccess) ce = cudaMemset(b->barrier, 0, 256);
    if (ce != cudaSuccess) {
        if (b->done) cudaEventDestroy(b->done);
        if (b->barrier) cudaFree(b->barrier);
        cudaStreamDestroy(b->stream);
        return cuda_fail(ce, "pbf_batch_create");
    }
    *out = b.release();
    return PBF_OK;
}

int pbf_batch_destroy(pbf_batch* b) {
    if (!b) return PBF_OK;
    {
        DeviceGuard dg(b->device);
        if (b->stream) cudaStreamSynchronize(b->stream);
        drop_graph(b);
        free_tables(b);
        for (auto& kv : b->tune) {
            if (kv.second.e0) cudaEventDestroy(kv.second.e0);
            if (kv.second.e1) cudaEventDestroy(kv.second.e1);
        }
        for (void* m : {b->wmem, b->smem, b->xmem, static_cast<void*>(b->off),
                        static_cast<void*>(b->d_bad), static_cast<void*>(b->barrier)})
            if (m) cudaFree(m);
        if (b->done) cudaEventDestroy(b->done);
        if (b->fork) cudaEventDestroy(b->fork);
        if (b->stream) cudaStreamDestroy(b->stream);
    }
    delete b;
    return PBF_OK;
}

int pbf_batch_step(pbf_batch* b, int nscenes, pbf_scene* const* scenes, const float* dt,
                   const int* nsteps) {
    int rc = check_args(b, nscenes, scenes, dt);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(b->mu);
    DeviceGuard dg(b->device);
    SceneLocks L;
    rc = lock_scenes(b, nscenes, scenes, L);
    if (rc) return rc;
    rc = wait_for_scenes(b, nscenes, scenes);
    if (!rc) rc = run_batch(b, nscenes, scenes, dt, nsteps);
    const int rc2 = release_scenes(b, nscenes, scenes);
    return rc ? rc : rc2;
}

int pbf_batch_step_timed(pbf_batch* b, int nscenes, pbf_scene* const* scenes, const float* dt,
                         const int* nsteps, float* ms_out) {
    int rc = check_args(b, nscenes, scenes, dt);
    if (rc) return rc;
    if (!ms_out) return fail(PBF_ERR_INVALID_ARG, "ms_out is NULL");
    *ms_out = 0.0f;
    std::lock_guard<std::mutex> lk(b->mu);
    DeviceGuard dg(b->device);
    SceneLocks L;
    rc = lock_scenes(b, nscenes, scenes, L);
    if (rc) return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    PBF_CUDA(cudaEventCreate(&e0));
    cudaError_t e = cudaEventCreate(&e1);
    rc = wait_for_scenes(b, nscenes, scenes);
    if (!rc && e == cudaSuccess) e = cudaEventRecord(e0, b->stream);
    if (!rc && e == cudaSuccess) rc = run_batch(b, nscenes, scenes, dt, nsteps);
    if (!rc && e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
    const int rc2 = release_scenes(b, nscenes, scenes);
    if (!rc && e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (!rc && e == cudaSuccess) e = cudaEventElapsedTime(ms_out, e0, e1);
    cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (rc) return rc;
    if (rc2) return rc2;
    if (e != cudaSuccess) return cuda_fail(e, "pbf_batch_step_timed");
    return batch_sync(b);
}

int pbf_batch_replay_timed(pbf_batch* b, int nscenes, pbf_scene* const* scenes,
                           const pbf_snapshot* const* seeds, const float* dt, int nsteps,
                           float* ms_out) {
    int rc = check_args(b, nscenes, scenes, dt);
    if (rc) return rc;
    if (!ms_out || (nscenes > 0 && !seeds)) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    if (nsteps < 0) return fail(PBF_ERR_INVALID_ARG, "nsteps must be >= 0");
    for (int k = 0; k < nscenes; ++k)
        if (!seeds[k]) return fail(PBF_ERR_INVALID_ARG, "a seed is NULL");
    *ms_out = 0.0f;
    std::lock_guard<std::mutex> lk(b->mu);
    DeviceGuard dg(b->device);
    SceneLocks L;
    rc = lock_scenes(b, nscenes, scenes, L);
    if (rc) return rc;
    rc = wait_for_scenes(b, nscenes, scenes);
    auto seeded_step = [&]() {
        for (int k = 0; k < nscenes; ++k) {
            const int r = restore_on(scenes[k], seeds[k], b->stream);
            if (r) return r;
        }
        return run_batch(b, nscenes, scenes, dt, nullptr);
    };
    if (!rc) rc = seeded_step();  // builds the graph outside the timed region
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (!rc && e == cudaSuccess) e = cudaEventRecord(e0, b->stream);
    for (int k = 0; k < nsteps && !rc && e == cudaSuccess; ++k) rc = seeded_step();
    if (!rc && e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
    const int rc2 = release_scenes(b, nscenes, scenes);
    if (!rc && e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (!rc && e == cudaSuccess) e = cudaEventElapsedTime(ms_out, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (rc) return rc;
    if (rc2) return rc2;
    if (e != cudaSuccess) return cuda_fail(e, "pbf_batch_replay_timed");
    return batch_sync(b);
}

int pbf_batch_set_persistent(pbf_batch* b, int on) {
    if (!b) return fail(PBF_ERR_INVALID_ARG, "batch is NULL");
    std::lock_guard<std::mutex> lk(b->mu);
    b->persistent = on != 0;
    return PBF_OK;
}

int pbf_batch_set_autotune(pbf_batch* b, int on) {
    if (!b) return fail(PBF_ERR_INVALID_ARG, "batch is NULL");
    std::lock_guard<std::mutex> lk(b->mu);
    DeviceGuard dg(b->device);
    b->autotune = on != 0;
    if (b->autotune && b->gpu.empty()) {
        cudaDeviceProp prop{};
        PBF_CUDA(cudaGetDeviceProperties(&prop, b->device));
        b->gpu = prop.name;
        b->cache_path = cache_file();
        load_tuning(b);
    }
    return PBF_OK;
}

int pbf_batch_tuning(const pbf_batch* b, int* block, int* persistent) {
    if (!b || !block || !persistent) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    *block = b->last.block;
    *persistent = b->last.persist;
    return PBF_OK;
}

int pbf_batch_sync(pbf_batch* b) {
    if (!b) return fail(PBF_ERR_INVALID_ARG, "batch is NULL");
    std::lock_guard<std::mutex> lk(b->mu);
    DeviceGuard dg(b->device);
    return batch_sync(b);
}

int pbf_batch_device_bytes(const pbf_batch* b, size_t* out) {
    if (!b || !out) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    *out = batch_bytes(b);
    return PBF_OK;
}

int pbf_batch_nonfinite(pbf_batch* b, int nscenes, int* out) {
    if (!b || (nscenes > 0 && !out)) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(b->mu);
    DeviceGuard dg(b->device);
    if (nscenes != b->bad_count)
        return fail(PBF_ERR_INVALID_ARG, "nscenes differs from the last batch call");
    if (nscenes == 0) return PBF_OK;
    std::vector<uint32_t> h((size_t)nscenes);
    PBF_CUDA(cudaMemcpyAsync(h.data(), b->d_bad, (size_t)nscenes * 4, cudaMemcpyDeviceToHost,
                             b->stream));
    PBF_CUDA(cudaStreamSynchronize(b->stream));
    for (int k = 0; k < nscenes; ++k) out[k] = h[k] ? 1 : 0;
    return PBF_OK;
}

int pbf_scene_device_bytes(const pbf_scene* s, size_t* out) {
    if (!s || !out) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
    *out = scene_device_bytes(s);
    return PBF_OK;
}

size_t pbf_state_bytes_per_particle(void) { return kStateBytesPerParticle; }

}  // extern "C"
