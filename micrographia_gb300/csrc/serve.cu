// The serving loop: simulation requests of different sizes and dimensions admitted against an
// HBM budget, their state resident on the device, stepped concurrently and streaming frames of
// observables back.
//
// Continuous batching, two ways:
// - Small requests (at most `lane_max_n` particles) of one dimension are stepped together in that
//   dimension's lane: one batch (gbmd_batch: the systems in one set of arrays, every force step a
//   single launch over all of them, 100-step graphs) advancing all its members a frame interval
//   at a time, then one frame pass for all of them (gbmd_batch_observe). A request admitted while
//   the lane runs joins it at the next interval boundary, and a finished one leaves there: the
//   lane re-packs its members' states (read back in one conversion) with the joiners' seeded
//   initial states into a new batch. Members share the lane's frame cadence and RDF shape; a
//   request that does not match them takes the other way.
// - Every other request is an engine with its own CUDA stream.
// Each turn of the loop enqueues the next interval of every lane and engine whose previous one has
// finished, so all admitted work overlaps on the GPU, and a request that arrives while others run
// is admitted as soon as the budget and a slot allow (a finished request frees both at once).
// Engines and batches are deterministic and step each system exactly as a plain engine does, so
// each request's final state is the same alone and in any mix, bit for bit, and its frames agree
// to rounding (a lane sums the same terms in another order).
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

// The small requests of one dimension, stepped together in one batch.
struct Lane {
    uint32_t dim = 2; // (lanes[1] is the 3D lane)
    gbmd_batch* b = nullptr;
    std::vector<Request> members; // in the batch's system order
    std::vector<Request> joining; // admitted, joining at the next interval boundary
    uint32_t frame_every = 0, rdf_bins = 0;
    double rdf_rmax = 0.0, skin = 0.3;
    cudaEvent_t done = nullptr;
    bool running = false;
    bool changed = false;        // members left: re-pack before the next interval
    std::vector<uint32_t> old_n; // the batch's systems' sizes, in its order
    std::vector<uint32_t> keep;  // the batch's systems that stay (indices into old_n)
    std::vector<gbmd_frame> frames;
    std::vector<uint64_t> rdf;
    bool empty() const { return members.empty() && joining.empty(); }
};

} // namespace

struct gbmd_server {
    uint64_t budget = 0, in_use = 0;
    uint32_t max_active = 64;
    int device = 0;
    uint64_t next_id = 1;
    uint64_t t0 = 0;
    uint32_t lane_max_n = 65536;
    std::deque<Request> pending;
    std::vector<Request> active;
    Lane lanes[2]; // 2D, 3D
    std::deque<gbmd_serve_frame> out;
    uint64_t admitted = 0, completed = 0, atom_steps = 0, lane_requests = 0, lane_repacks = 0;
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

// Requests holding a slot: engines, lane members and lane joiners.
size_t held(const gbmd_server* sv) {
    size_t k = sv->active.size();
    for (const Lane& L : sv->lanes) k += L.members.size() + L.joining.size();
    return k;
}

// Whether request r goes into its dimension's lane: small enough, a frame cadence that divides its
// steps, and (when the lane holds members) the lane's cadence and RDF shape.
bool lane_takes(const gbmd_server* sv, const Request& r) {
    const gbmd_serve_request& q = r.spec;
    if (q.init.n > sv->lane_max_n || q.frame_every == 0 || q.steps % q.frame_every != 0) return false;
    const Lane& L = sv->lanes[q.sys.dim == 2 ? 0 : 1];
    if (L.empty()) return true;
    return q.frame_every == L.frame_every && std::min<uint32_t>(q.rdf_bins, GBMD_SERVE_RDF_BINS) == L.rdf_bins &&
           (q.rdf_rmax > 0 ? q.rdf_rmax : 5.0) == L.rdf_rmax;
}

// A lane's interval has finished: a frame for each member, then the members that are done leave.
int lane_collect(gbmd_server* sv, Lane& L) {
    L.running = false;
    const uint32_t K = (uint32_t)L.members.size();
    L.frames.assign(K, gbmd_frame{});
    L.rdf.assign((size_t)K * L.rdf_bins, 0);
    GBMD_TRY(gbmd_batch_observe_end(L.b, L.frames.data(), L.rdf_bins ? L.rdf.data() : nullptr));
    bool any_last = false;
    for (auto& m : L.members) any_last = any_last || m.steps_done >= m.spec.steps || m.cancelled;
    std::vector<int64_t> pos;
    std::vector<int32_t> vel;
    std::vector<uint32_t> sp;
    if (any_last) { // final states, for the hashes (one conversion for the whole batch)
        size_t N = 0;
        for (auto& m : L.members) N += m.spec.init.n;
        pos.resize(N * L.dim);
        vel.resize(N * L.dim);
        sp.resize(N);
        GBMD_TRY(gbmd_batch_read_all(L.b, pos.data(), vel.data(), sp.data()));
    }
    const uint64_t now = now_ns() - sv->t0;
    size_t off = 0;
    std::vector<Request> stay;
    L.old_n.clear();
    L.keep.clear();
    for (uint32_t k = 0; k < K; k++) {
        Request& m = L.members[k];
        gbmd_serve_frame f;
        std::memset(&f, 0, sizeof(f));
        f.request = m.id;
        f.index = m.frames++;
        f.frame = L.frames[k];
        f.frame.step = m.steps_done;
        if (L.rdf_bins) std::memcpy(f.rdf, L.rdf.data() + (size_t)k * L.rdf_bins, (size_t)L.rdf_bins * 8);
        const bool last = m.steps_done >= m.spec.steps || m.cancelled;
        f.last = last ? 1u : 0u;
        if (last) f.state_hash = gbmd_hash_state(L.dim, pos.data() + off * L.dim, vel.data() + off * L.dim, sp.data() + off, m.spec.init.n);
        f.ready_ns = now;
        sv->out.push_back(f);
        off += m.spec.init.n;
        L.old_n.push_back(m.spec.init.n);
        if (last) {
            sv->completed++;
            sv->in_use -= m.bytes;
            L.changed = true;
        } else {
            L.keep.push_back(k);
            stay.push_back(m);
        }
    }
    L.members.swap(stay);
    return GBMD_OK;
}

// Start a lane's next interval, re-packing its batch first when members left or are joining.
// The new batch is built before the old one is freed: if building fails, the lane keeps its
// batch, members and joiners, and the next poll tries again.
int lane_start(gbmd_server* sv, Lane& L) {
    if (L.running) return GBMD_OK;
    for (size_t q = 0; q < L.joining.size();) { // cancelled before it started: it leaves with no frame
        if (L.joining[q].cancelled) {
            sv->completed++;
            sv->in_use -= L.joining[q].bytes;
            L.joining.erase(L.joining.begin() + (long)q);
            L.changed = true;
        } else {
            q++;
        }
    }
    if (!L.joining.empty() || L.changed) {
        // the states to carry over: the survivors, picked out of the old batch by their index in
        // it; then the joiners. Each keeps its own step clock (its steps so far).
        std::vector<gbmd_system> systems;
        std::vector<uint32_t> offsets(1, 0);
        std::vector<int64_t> pos;
        std::vector<int32_t> vel;
        std::vector<uint32_t> sp;
        std::vector<Request> next;
        if (L.b && !L.members.empty()) {
            std::vector<size_t> first(L.old_n.size() + 1, 0);
            for (size_t k = 0; k < L.old_n.size(); k++) first[k + 1] = first[k] + L.old_n[k];
            const size_t N = first.back();
            std::vector<int64_t> ap(N * L.dim);
            std::vector<int32_t> av(N * L.dim);
            std::vector<uint32_t> as(N);
            GBMD_TRY(gbmd_batch_read_all(L.b, ap.data(), av.data(), as.data()));
            for (size_t q = 0; q < L.keep.size(); q++) { // the survivors, in order
                const size_t o = first[L.keep[q]], n = L.old_n[L.keep[q]];
                systems.push_back(L.members[q].spec.sys);
                pos.insert(pos.end(), ap.begin() + o * L.dim, ap.begin() + (o + n) * L.dim);
                vel.insert(vel.end(), av.begin() + o * L.dim, av.begin() + (o + n) * L.dim);
                sp.insert(sp.end(), as.begin() + o, as.begin() + o + n);
                offsets.push_back(offsets.back() + (uint32_t)n);
                next.push_back(L.members[q]);
            }
        }
        for (auto& r : L.joining) { // the joiners' seeded initial states
            const size_t n = r.spec.init.n, o = pos.size() / L.dim;
            pos.resize((o + n) * L.dim);
            vel.resize((o + n) * L.dim);
            sp.resize(o + n);
            GBMD_TRY(gbmd_init_state(&r.spec.sys, &r.spec.init, pos.data() + o * L.dim, vel.data() + o * L.dim, sp.data() + o));
            systems.push_back(r.spec.sys);
            offsets.push_back(offsets.back() + (uint32_t)n);
            next.push_back(r);
        }
        gbmd_batch* nb = nullptr;
        if (!next.empty()) {
            gbmd_options o{};
            o.mode = GBMD_MODE_VERLET;
            o.skin = L.skin;
            o.device = sv->device;
            o.block_steps = L.frame_every;
            GBMD_TRY(gbmd_batch_create(systems.data(), (uint32_t)systems.size(), offsets.data(), pos.data(), vel.data(), sp.data(), &o, &nb));
            std::vector<uint32_t> clocks;
            for (auto& m : next) clocks.push_back((uint32_t)m.steps_done);
            const int rc = gbmd_batch_set_clocks(nb, clocks.data());
            if (rc != GBMD_OK) {
                gbmd_batch_destroy(nb);
                return rc;
            }
            sv->lane_repacks++;
        }
        if (L.b) gbmd_batch_destroy(L.b);
        L.b = nb;
        L.members.swap(next);
        L.joining.clear();
        L.changed = false;
        // the new batch's systems are the members, in order, all kept until the next interval ends
        L.old_n.clear();
        L.keep.clear();
        for (size_t q = 0; q < L.members.size(); q++) {
            L.old_n.push_back(L.members[q].spec.init.n);
            L.keep.push_back((uint32_t)q);
        }
    }
    if (L.members.empty()) return GBMD_OK;
    if (!L.done) GBMD_CUDA_TRY(cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming));
    GBMD_TRY(gbmd_batch_step(L.b, L.frame_every));
    GBMD_TRY(gbmd_batch_observe_begin(L.b, L.rdf_bins, L.rdf_rmax));
    void* st = nullptr;
    GBMD_TRY(gbmd_batch_stream(L.b, &st));
    GBMD_CUDA_TRY(cudaEventRecord(L.done, (cudaStream_t)st));
    for (auto& m : L.members) {
        m.steps_done += L.frame_every;
        sv->atom_steps += L.frame_every * (uint64_t)m.spec.init.n;
    }
    L.running = true;
    return GBMD_OK;
}

int admit(gbmd_server* sv) {
    while (!sv->pending.empty() && held(sv) < sv->max_active) {
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
        if (lane_takes(sv, r)) {
            Lane& L = sv->lanes[r.spec.sys.dim == 2 ? 0 : 1];
            if (L.empty()) { // the first member sets the lane's frame cadence and RDF shape
                L.frame_every = r.spec.frame_every;
                L.rdf_bins = std::min<uint32_t>(r.spec.rdf_bins, GBMD_SERVE_RDF_BINS);
                L.rdf_rmax = r.spec.rdf_rmax > 0 ? r.spec.rdf_rmax : 5.0;
                L.skin = r.spec.skin > 0 ? r.spec.skin : 0.3;
            }
            r.bytes = need;
            sv->in_use += need;
            sv->admitted++;
            sv->lane_requests++;
            L.joining.push_back(r);
            continue;
        }
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
    sv->lanes[0].dim = 2;
    sv->lanes[1].dim = 3;
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
    for (Lane& L : sv->lanes) // the lanes: a finished interval's frames, leavers out
        if (L.running && cudaEventQuery(L.done) == cudaSuccess) GBMD_TRY(lane_collect(sv, L));
    GBMD_TRY(admit(sv));
    for (Lane& L : sv->lanes) GBMD_TRY(lane_start(sv, L)); // joiners in, the next interval
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
    for (Lane& L : sv->lanes) {
        for (auto& r : L.members)
            if (r.id == id) {
                r.cancelled = true; // leaves the lane after its interval in flight finishes
                return GBMD_OK;
            }
        for (auto& r : L.joining)
            if (r.id == id) {
                r.cancelled = true;
                return GBMD_OK;
            }
    }
    return fail(GBMD_E_NOTFOUND, "no such request");
}

int gbmd_serve_stats(gbmd_server* sv, gbmd_serve_stats_t* st) {
    if (!sv || !st) return fail(GBMD_E_INVALID, "null argument");
    st->pending = (uint32_t)sv->pending.size();
    st->active = (uint32_t)held(sv);
    st->admitted = sv->admitted;
    st->completed = sv->completed;
    st->bytes_in_use = sv->in_use;
    st->budget = sv->budget;
    st->atom_steps = sv->atom_steps;
    st->lane_requests = sv->lane_requests;
    st->lane_repacks = sv->lane_repacks;
    return GBMD_OK;
}

int gbmd_serve_set_lanes(gbmd_server* sv, uint32_t lane_max_n) {
    if (!sv) return fail(GBMD_E_INVALID, "null server");
    for (const Lane& L : sv->lanes)
        if (!L.empty()) return fail(GBMD_E_INVALID, "the lanes hold requests: set them before submitting");
    sv->lane_max_n = lane_max_n;
    return GBMD_OK;
}

int gbmd_serve_destroy(gbmd_server* sv) {
    if (!sv) return GBMD_OK;
    while (!sv->active.empty()) {
        if (sv->active.back().e) gbmd_sync(sv->active.back().e);
        retire(sv, sv->active.size() - 1);
    }
    for (Lane& L : sv->lanes) {
        if (L.b) {
            if (L.running) gbmd_batch_observe_end(L.b, nullptr, nullptr);
            gbmd_batch_destroy(L.b);
        }
        if (L.done) cudaEventDestroy(L.done);
    }
    delete sv;
    return GBMD_OK;
}

uint64_t gbmd_serve_estimate_bytes(const gbmd_system* sys, uint32_t n, double skin) {
    return sys ? estimate_bytes(*sys, n, skin > 0 ? skin : 0.3) : 0;
}

} // extern "C"
