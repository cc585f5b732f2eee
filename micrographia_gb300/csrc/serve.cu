// The serving loop: simulation requests of different sizes and dimensions admitted against an
// HBM budget, their state resident on the device, stepped concurrently and streaming frames of
// observables back.
//
// Continuous batching: every admitted request is an engine with its own CUDA stream; each turn
// of the loop enqueues the next frame interval of every request whose previous interval has
// finished, so the work of all admitted requests overlaps on the GPU, and a request that arrives
// while others run is admitted as soon as the budget and a slot allow (a finished request frees
// both at once). Engines are deterministic, so each request's frames and final state are the
// same alone and in any mix.
//
// The reference has no serving layer (its engines run one scenario per page,
// crates/wasm/src/sims.rs:29-516); this is the served form of the same engine.
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

#include "common.cuh"
#include "engine.cuh"

using namespace gbmd;

namespace {

uint64_t now_ns() {
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
    uint64_t id = 0;
    gbmd_serve_request spec{};
    gbmd_engine* e = nullptr;
    cudaEvent_t done = nullptr;
    uint64_t steps_done = 0;
    uint32_t frames = 0;
    uint64_t bytes = 0;
    bool running = false; // a frame interval is in flight
    bool cancelled = false;
};

} // namespace

struct gbmd_server {
    uint64_t budget = 0, in_use = 0;
    uint32_t max_active = 64;
    int device = 0;
    uint64_t next_id = 1;
    uint64_t t0 = 0;
    std::deque<Request> pending;
    std::vector<Request> active;
    std::deque<gbmd_serve_frame> out;
    uint64_t admitted = 0, completed = 0, atom_steps = 0;
};

namespace {

// Device bytes an engine for `n` particles of this system will allocate (create_common's
// buffers): positions x2, scratch, reference and quotient records, velocities, species, ids,
// sort keys/values x2, histograms, cell starts, the list, and per-particle helper arrays.
uint64_t estimate_bytes(const gbmd_system& s, uint32_t n, double skin) {
    double D = s.dim, rec = s.dim == 2 ? 16 : 32;
    double r = 0.0;
    for (uint32_t k = 0; k < s.nspecies * s.nspecies; k++) r = std::max(r, s.pairs[k].rc);
    r += skin;
    double vol = 1.0;
    for (uint32_t a = 0; a < s.dim; a++) vol *= (double)s.box_len[a] / 4294967296.0;
    double sphere = s.dim == 2 ? M_PI * r * r : 4.0 / 3.0 * M_PI * r * r * r;
    double cap = std::ceil(sphere * std::max(2.0 * n / vol, 1.2)) + 8;
    double cells = vol / std::pow(r, s.dim);
    double per = 4 * rec + 16 + 16 + 16 + 3 * 4 * D + 7 * 4 + 8 * D + 8;
    return (uint64_t)(n * per + n * 4.0 * (std::ceil(cap / 4) * 4) + cells * 4 + (1 << 20));
}

// Enqueue the next frame interval: its steps, then the frame's kernels and copies into pinned
// memory (gbmd_observe_begin), then the completion event. Nothing here waits on the device.
int start_interval(gbmd_server* sv, Request& r) {
    uint64_t left = r.spec.steps - r.steps_done;
    uint64_t k = std::min<uint64_t>(left, r.spec.frame_every ? r.spec.frame_every : left);
    GBMD_TRY(gbmd_step(r.e, k));
    const uint32_t bins = std::min<uint32_t>(r.spec.rdf_bins, GBMD_SERVE_RDF_BINS);
    GBMD_TRY(gbmd_observe_begin(r.e, bins, r.spec.rdf_rmax > 0 ? r.spec.rdf_rmax : 5.0, 0, 0));
    void* st = nullptr;
    GBMD_TRY(gbmd_stream(r.e, &st));
    GBMD_CUDA_TRY(cudaEventRecord(r.done, (cudaStream_t)st));
    r.steps_done += k;
    r.running = true;
    sv->atom_steps += k * (uint64_t)r.spec.init.n;
    return GBMD_OK;
}

int admit(gbmd_server* sv) {
    while (!sv->pending.empty() && sv->active.size() < sv->max_active) {
        Request& q = sv->pending.front();
        if (q.cancelled) {
            sv->pending.pop_front();
            continue;
        }
        uint64_t need = estimate_bytes(q.spec.sys, q.spec.init.n, q.spec.skin > 0 ? q.spec.skin : 0.3);
        if (need > sv->budget) {
            uint64_t id = q.id;
            sv->pending.pop_front();
            return fail(GBMD_E_BUDGET, "request " + std::to_string(id) + " needs more device memory than the whole budget");
        }
        if (sv->in_use + need > sv->budget) break; // wait for memory (first come, first served)
        Request r = q;
        sv->pending.pop_front();
        gbmd_options o{};
        o.mode = GBMD_MODE_VERLET;
        o.skin = r.spec.skin > 0 ? r.spec.skin : 0.3;
        o.device = sv->device;
        o.block_steps = r.spec.frame_every ? r.spec.frame_every : 0;
        GBMD_TRY(gbmd_create_seeded(&r.spec.sys, &r.spec.init, &o, &r.e));
        GBMD_CUDA_TRY(cudaEventCreateWithFlags(&r.done, cudaEventDisableTiming));
        r.bytes = need;
        sv->in_use += need;
        sv->admitted++;
        GBMD_TRY(start_interval(sv, r));
        sv->active.push_back(r);
    }
    return GBMD_OK;
}

int emit_frame(gbmd_server* sv, Request& r) {
    gbmd_serve_frame f;
    std::memset(&f, 0, sizeof(f));
    f.request = r.id;
    f.index = r.frames++;
    // the interval's event has completed: the frame is already in pinned memory
    GBMD_TRY(gbmd_observe_end(r.e, &f.frame, f.rdf, nullptr));
    f.last = r.steps_done >= r.spec.steps ? 1u : 0u;
    if (f.last) GBMD_TRY(gbmd_state_hash(r.e, &f.state_hash));
    f.ready_ns = now_ns() - sv->t0;
    sv->out.push_back(f);
    return GBMD_OK;
}

void retire(gbmd_server* sv, size_t k) {
    Request& r = sv->active[k];
    if (r.done) cudaEventDestroy(r.done);
    gbmd_destroy(r.e);
    sv->in_use -= r.bytes;
    sv->active.erase(sv->active.begin() + (long)k);
}

} // namespace

extern "C" {

int gbmd_serve_create(uint64_t hbm_budget_bytes, uint32_t max_active, int32_t device, gbmd_server** out) {
    if (!out || hbm_budget_bytes == 0) return fail(GBMD_E_INVALID, "a server needs a positive HBM budget");
    auto* sv = new gbmd_server;
    sv->budget = hbm_budget_bytes;
    sv->max_active = max_active ? max_active : 64;
    sv->device = device;
    sv->t0 = now_ns();
    *out = sv;
    return GBMD_OK;
}

int gbmd_serve_submit(gbmd_server* sv, const gbmd_serve_request* req, uint64_t* id) {
    if (!sv || !req) return fail(GBMD_E_INVALID, "null argument");
    GBMD_TRY(validate_system(req->sys, req->init.n));
    if (req->init.n == 0 || req->steps == 0) return fail(GBMD_E_INVALID, "a request needs particles and steps");
    if ((req->sys.periodic & ((1u << req->sys.dim) - 1u)) != ((1u << req->sys.dim) - 1u))
        return fail(GBMD_E_UNSUPPORTED, "served requests are periodic systems");
    Request r;
    r.id = sv->next_id++;
    r.spec = *req;
    sv->pending.push_back(r);
    if (id) *id = r.id;
    return GBMD_OK;
}

int gbmd_serve_poll(gbmd_server* sv, gbmd_serve_frame* frames, uint32_t cap, uint32_t* count) {
    if (!sv || !count || (cap && !frames)) return fail(GBMD_E_INVALID, "null argument");
    *count = 0;
    // collect finished intervals: a frame each, then the next interval or retirement
    for (size_t k = 0; k < sv->active.size();) {
        Request& r = sv->active[k];
        if (r.running && cudaEventQuery(r.done) == cudaSuccess) {
            r.running = false;
            GBMD_TRY(emit_frame(sv, r));
            if (r.steps_done >= r.spec.steps || r.cancelled) {
                sv->completed++;
                retire(sv, k);
                continue;
            }
            GBMD_TRY(start_interval(sv, r));
        }
        k++;
    }
    GBMD_TRY(admit(sv));
    while (*count < cap && !sv->out.empty()) {
        frames[(*count)++] = sv->out.front();
        sv->out.pop_front();
    }
    return GBMD_OK;
}

int gbmd_serve_cancel(gbmd_server* sv, uint64_t id) {
    if (!sv) return fail(GBMD_E_INVALID, "null server");
    for (auto& r : sv->pending)
        if (r.id == id) {
            r.cancelled = true;
            return GBMD_OK;
        }
    for (size_t k = 0; k < sv->active.size(); k++)
        if (sv->active[k].id == id) {
            sv->active[k].cancelled = true; // retired after its interval in flight finishes
            return GBMD_OK;
        }
    return fail(GBMD_E_NOTFOUND, "no such request");
}

int gbmd_serve_stats(gbmd_server* sv, gbmd_serve_stats_t* st) {
    if (!sv || !st) return fail(GBMD_E_INVALID, "null argument");
    st->pending = (uint32_t)sv->pending.size();
    st->active = (uint32_t)sv->active.size();
    st->admitted = sv->admitted;
    st->completed = sv->completed;
    st->bytes_in_use = sv->in_use;
    st->budget = sv->budget;
    st->atom_steps = sv->atom_steps;
    return GBMD_OK;
}

int gbmd_serve_destroy(gbmd_server* sv) {
    if (!sv) return GBMD_OK;
    while (!sv->active.empty()) {
        if (sv->active.back().e) gbmd_sync(sv->active.back().e);
        retire(sv, sv->active.size() - 1);
    }
    delete sv;
    return GBMD_OK;
}

uint64_t gbmd_serve_estimate_bytes(const gbmd_system* sys, uint32_t n, double skin) {
    return sys ? estimate_bytes(*sys, n, skin > 0 ? skin : 0.3) : 0;
}

} // extern "C"
