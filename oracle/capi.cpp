// ORACLE — test infrastructure only: a C API over oracle.hpp for the Python parity tests and the
// CPU baseline. The engine never links or calls it.
#include <cstring>
#include <memory>

#include "oracle.hpp"

using namespace oracle;

namespace {

State make_state(int dim, const int64_t* pos, const int32_t* vel, const uint32_t* species, uint64_t n) {
    State s;
    s.dim = dim;
    s.pos.assign(pos, pos + dim * n);
    s.vel.assign(vel, vel + dim * n);
    s.species.assign(species, species + n);
    return s;
}
State make_state_pos(int dim, const int64_t* pos, const uint32_t* species, uint64_t n) {
    State s;
    s.dim = dim;
    s.pos.assign(pos, pos + dim * n);
    s.vel.assign(dim * n, 0);
    if (species) s.species.assign(species, species + n);
    else s.species.assign(n, 0);
    return s;
}

struct Engine {
    std::unique_ptr<IntEngine<float>> f32;
    std::unique_ptr<IntEngine<double>> f64;
    State& state() { return f32 ? f32->state : f64->state; }
};

} // namespace

extern "C" {

// ---- fixed point, RNG, libm restatement
int oracle_sep_f32(int64_t d, float* out) { return sep_f32(d, out) ? 1 : 0; }
float oracle_sep_near(int64_t d) { return sep_near_f32(d); }
void oracle_threefry(uint32_t c0, uint32_t c1, uint32_t k0, uint32_t k1, uint32_t rounds, uint32_t* out) {
    auto r = threefry2x32_rounds({c0, c1}, {k0, k1}, rounds);
    out[0] = r[0];
    out[1] = r[1];
}
double oracle_uniform(uint64_t seed, uint32_t stream, uint32_t i) { return uniform(seed, stream, i); }
double oracle_normal(uint64_t seed, uint32_t stream, uint32_t i) { return normal(seed, stream, i); }
double oracle_log(double x) { return fdlibm::log(x); }
double oracle_cos(double x) { return fdlibm::cos(x); }
double oracle_sin(double x) { return fdlibm::sin(x); }
// fdlibm's ln, cos and sin at n arguments: out[3 i], out[3 i + 1], out[3 i + 2].
void oracle_fdlibm_many(const double* x, uint64_t n, double* out) {
    for (uint64_t i = 0; i < n; i++) {
        out[3 * i] = fdlibm::log(x[i]);
        out[3 * i + 1] = fdlibm::cos(x[i]);
        out[3 * i + 2] = fdlibm::sin(x[i]);
    }
}
// How often the device's fdlibm ln, cos and sin and the platform libm (what the reference's f64
// methods call on a native build) round differently on the heat bath's own arguments, and how
// often that changes a redrawn velocity: n 2D draws as walls::andersen makes them (u1 = 1 - U,
// a = 2 pi U', Threefry on (k, 0) under the key of `seed`), each component rounded by
// to_step_displacement at kT/m = t_over_m and step dt. out: ln, cos, sin disagreements, then the
// draws whose x or y step displacement differs.
void oracle_libm_compare(uint64_t n, uint64_t seed, double t_over_m, double dt, uint64_t* out) {
    const std::array<uint32_t, 2> key{(uint32_t)seed, (uint32_t)(seed >> 32) ^ STREAM_THERMO};
    uint64_t c[4] = {0, 0, 0, 0};
    const double sd = std::sqrt(t_over_m);
    auto step = [&](double u) { return sat_i32(std::round(u * dt * 4294967296.0)); };
    for (uint64_t k = 0; k < n; k++) {
        const auto r = threefry2x32({(uint32_t)k, (uint32_t)(k >> 32)}, key);
        const auto r2 = threefry2x32({(uint32_t)k, (uint32_t)(k >> 32)}, {key[0], key[1] ^ 1u});
        const double u1 = 1.0 - to_unit_f64({r[1], 0}), a = TAU * to_unit_f64({r2[0], 0});
        const double lf = fdlibm::log(u1), lg = std::log(u1);
        const double cf = fdlibm::cos(a), cg = std::cos(a), sf = fdlibm::sin(a), sg = std::sin(a);
        c[0] += lf != lg;
        c[1] += cf != cg;
        c[2] += sf != sg;
        const double rf = std::sqrt(-2.0 * lf), rg = std::sqrt(-2.0 * lg);
        c[3] += step(sd * rf * cf) != step(sd * rg * cg) || step(sd * rf * sf) != step(sd * rg * sg);
    }
    for (int q = 0; q < 4; q++) out[q] = c[q];
}
int64_t oracle_to_fixed(double x) { return to_fixed(x); }

// ---- System helpers
void oracle_box_for(uint64_t n, double density, double aspect, int64_t* out) {
    auto b = box_for(n, density, aspect);
    out[0] = b[0];
    out[1] = b[1];
}
void oracle_cube_for(uint64_t n, double density, int64_t* out) {
    auto b = cube_for(n, density);
    for (int a = 0; a < 3; a++) out[a] = b[a];
}
void oracle_fcc_cells(uint64_t n, const int64_t* box, uint64_t* out) {
    auto c = fcc_cells(n, {box[0], box[1], box[2]});
    for (int a = 0; a < 3; a++) out[a] = c[a];
}
int oracle_cells_for(const gbmd_system* csys, double r, uint32_t* out) {
    try {
        auto c = System::from_c(*csys).cells_for(r);
        for (int a = 0; a < 3; a++) out[a] = c[a];
        return 0;
    } catch (...) {
        return -1;
    }
}
double oracle_wca_rc(void) { return Pair::wca().rc; }
double oracle_pair_shift(double eps, double sigma, double rc) { return Pair{eps, sigma, rc}.shift(); }

// ---- initial conditions (md-core init.rs / three.rs and this engine's recipes)
void oracle_lattice(uint64_t n, const int64_t* box, double jitter, uint64_t seed, int64_t* pos) {
    auto p = lattice(n, {box[0], box[1]}, jitter, seed);
    std::memcpy(pos, p.data(), p.size() * 8);
}
void oracle_fcc(uint64_t n, const int64_t* box, const uint64_t* cells, double jitter, uint64_t seed, int64_t* pos) {
    auto p = fcc(n, {box[0], box[1], box[2]}, {cells[0], cells[1], cells[2]}, jitter, seed);
    std::memcpy(pos, p.data(), p.size() * 8);
}
void oracle_maxwell(const gbmd_system* csys, const uint32_t* species, uint64_t n, double t, uint64_t seed, int32_t* vel) {
    System sys = System::from_c(*csys);
    std::vector<uint32_t> sp(species, species + n);
    auto v = maxwell(sys, sp, t, seed);
    std::memcpy(vel, v.data(), v.size() * 4);
}
void oracle_zero_velocity_sum(const gbmd_system* csys, const uint32_t* species, uint64_t n, int32_t* vel) {
    System sys = System::from_c(*csys);
    std::vector<uint32_t> sp(species, species + n);
    std::vector<int32_t> v(vel, vel + sys.dim * n);
    zero_velocity_sum(sys, sp, v, sys.dim == 3);
    std::memcpy(vel, v.data(), v.size() * 4);
}
void oracle_set_temperature(const gbmd_system* csys, int32_t* vel, const uint32_t* species, uint64_t n, double t, int exact) {
    System sys = System::from_c(*csys);
    State s;
    s.dim = sys.dim;
    s.vel.assign(vel, vel + sys.dim * n);
    s.species.assign(species, species + n);
    s.pos.assign(sys.dim * n, 0);
    if (exact) rescale_temperature(s, sys, t);
    else set_temperature(s, sys, t);
    std::memcpy(vel, s.vel.data(), s.vel.size() * 4);
}
double oracle_exact_kinetic(const gbmd_system* csys, const int32_t* vel, const uint32_t* species, uint64_t n) {
    System sys = System::from_c(*csys);
    State s;
    s.dim = sys.dim;
    s.vel.assign(vel, vel + sys.dim * n);
    s.species.assign(species, species + n);
    return exact_half_step_kinetic(sys, s);
}
double oracle_half_step_kinetic(const gbmd_system* csys, const int32_t* vel, const uint32_t* species, uint64_t n) {
    System sys = System::from_c(*csys);
    State s;
    s.dim = sys.dim;
    s.vel.assign(vel, vel + sys.dim * n);
    s.species.assign(species, species + n);
    return half_step_kinetic(sys, s);
}
// The recipes of gbmd_init_state, restated on the CPU.
int oracle_init(const gbmd_system* csys, const gbmd_init* spec, int64_t* pos, int32_t* vel, uint32_t* species) {
    try {
        System sys = System::from_c(*csys);
        size_t n = spec->n;
        State st;
        switch (spec->recipe) {
            case GBMD_INIT_FLUID: {
                // init::fluid (init.rs:105-121): on an axis with walls the lattice keeps 1 sigma
                // clear of them
                st.dim = 2;
                int64_t inner[2];
                for (int a = 0; a < 2; a++) inner[a] = sys.periodic(a) ? sys.box[a] : sys.box[a] - to_fixed(2.0);
                st.pos = lattice(n, {inner[0], inner[1]}, spec->jitter, spec->seed);
                for (size_t i = 0; i < n; i++)
                    for (int a = 0; a < 2; a++)
                        if (!sys.periodic(a)) st.pos[2 * i + a] += to_fixed(1.0);
                st.species.assign(n, 0);
                st.vel = maxwell(sys, st.species, spec->t, spec->seed);
                break;
            }
            case GBMD_INIT_TRIANGULAR: {
                st.dim = 2;
                st.pos = triangular(n, {sys.box[0], sys.box[1]}, {0, 0}, {sys.box[0], sys.box[1]}, spec->jitter, spec->seed, 0);
                st.species.assign(n, 0);
                st.vel = maxwell(sys, st.species, spec->t, spec->seed);
                break;
            }
            case GBMD_INIT_FCC: {
                st.dim = 3;
                std::array<int64_t, 3> b{sys.box[0], sys.box[1], sys.box[2]};
                st.pos = fcc(n, b, fcc_cells(n, b), spec->jitter, spec->seed);
                st.species.assign(n, 0);
                st.vel = maxwell(sys, st.species, spec->t, spec->seed);
                break;
            }
            case GBMD_INIT_SLAB:
                st = slab(sys, n, spec->rho_liquid, spec->rho_vapour, spec->slab_frac, spec->t, spec->jitter, spec->seed);
                break;
            default:
                return -1;
        }
        if (pos) std::memcpy(pos, st.pos.data(), st.pos.size() * 8);
        if (vel) std::memcpy(vel, st.vel.data(), st.vel.size() * 4);
        if (species) std::memcpy(species, st.species.data(), st.species.size() * 4);
        return 0;
    } catch (...) {
        return -1;
    }
}

// ---- cells and Verlet lists
int oracle_cell_list(const gbmd_system* csys, const int64_t* pos, uint64_t n, const uint32_t* dims, uint32_t* keys, uint32_t* start,
                     uint32_t* items) {
    System sys = System::from_c(*csys);
    State s = make_state_pos(sys.dim, pos, nullptr, n);
    CellList cl = build_cells(sys, s, {dims[0], dims[1], dims[2]});
    std::memcpy(keys, cl.keys.data(), n * 4);
    std::memcpy(start, cl.start.data(), cl.start.size() * 4);
    std::memcpy(items, cl.items.data(), n * 4);
    return 0;
}
uint32_t oracle_verlet_cap(const gbmd_system* csys, uint64_t n, double skin) { return verlet_cap(System::from_c(*csys), n, skin); }
// Lists packed particle by particle (sorted indices); returns the total, or -1 past `cap` entries.
int64_t oracle_verlet_list(const gbmd_system* csys, const int64_t* pos, const uint32_t* species, uint64_t n, double skin, uint32_t* counts,
                           uint32_t* nbr, uint64_t cap) {
    System sys = System::from_c(*csys);
    State s = make_state_pos(sys.dim, pos, species, n);
    auto lists = verlet_lists(sys, s, skin);
    uint64_t off = 0;
    for (size_t i = 0; i < n; i++) {
        counts[i] = (uint32_t)lists[i].size();
        if (off + lists[i].size() > cap) return -1;
        std::memcpy(nbr + off, lists[i].data(), lists[i].size() * 4);
        off += lists[i].size();
    }
    return (int64_t)off;
}

// The lists of the particles idx[0..m) only, packed like oracle_verlet_list.
int64_t oracle_verlet_list_of(const gbmd_system* csys, const int64_t* pos, const uint32_t* species, uint64_t n, double skin,
                              const uint32_t* idx, uint64_t m, int threads, uint32_t* counts, uint32_t* nbr, uint64_t cap) {
    System sys = System::from_c(*csys);
    State s = make_state_pos(sys.dim, pos, species, n);
    auto lists = verlet_lists_of(sys, s, skin, idx, m, threads > 0 ? threads : 1);
    uint64_t off = 0;
    for (size_t q = 0; q < m; q++) {
        counts[q] = (uint32_t)lists[q].size();
        if (off + lists[q].size() > cap) return -1;
        std::memcpy(nbr + off, lists[q].data(), lists[q].size() * 4);
        off += lists[q].size();
    }
    return (int64_t)off;
}

// ---- engines
void* oracle_engine_create(const gbmd_system* csys, const int64_t* pos, const int32_t* vel, const uint32_t* species, uint64_t n, int use_f64,
                           int fast, int int_tables, int threads) {
    try {
        System sys = System::from_c(*csys);
        State s = make_state(sys.dim, pos, vel, species, n);
        auto* e = new Engine;
        if (use_f64) {
            e->f64.reset(new IntEngine<double>(sys, s));
            e->f64->fast = fast != 0;
            e->f64->threads = threads > 0 ? threads : 1;
            if (int_tables) e->f64->use_integer_tables();
        } else {
            e->f32.reset(new IntEngine<float>(sys, s));
            e->f32->fast = fast != 0;
            e->f32->threads = threads > 0 ? threads : 1;
            if (int_tables) e->f32->use_integer_tables();
        }
        return e;
    } catch (...) {
        return nullptr;
    }
}
void oracle_engine_destroy(void* h) { delete (Engine*)h; }
// The half-shell 3D pair loop (IntEngine::half3): same kicks, about half the work.
void oracle_engine_set_half3(void* h, int on) {
    Engine* e = (Engine*)h;
    if (e->f32) e->f32->half3 = on != 0;
    else e->f64->half3 = on != 0;
}
void oracle_engine_step(void* h, uint64_t steps) {
    Engine* e = (Engine*)h;
    if (e->f32) e->f32->step(steps);
    else e->f64->step(steps);
}
void oracle_engine_reverse(void* h) {
    Engine* e = (Engine*)h;
    if (e->f32) e->f32->reverse();
    else e->f64->reverse();
}
double oracle_engine_kicks(void* h, int32_t* kicks) {
    Engine* e = (Engine*)h;
    std::vector<int32_t> k;
    double pe = e->f32 ? e->f32->forces(k) : e->f64->forces(k);
    std::memcpy(kicks, k.data(), k.size() * 4);
    return pe;
}
// The kicks IntEngine's forces() gives the particles idx[0..m) of the engine's state (the
// reference loop on those particles only).
void oracle_engine_kicks_of(void* h, const uint32_t* idx, uint64_t m, int32_t* kicks) {
    Engine* e = (Engine*)h;
    if (e->f32) e->f32->forces_of(idx, m, kicks);
    else e->f64->forces_of(idx, m, kicks);
}
void oracle_engine_state(void* h, int64_t* pos, int32_t* vel, uint32_t* species) {
    State& s = ((Engine*)h)->state();
    if (pos) std::memcpy(pos, s.pos.data(), s.pos.size() * 8);
    if (vel) std::memcpy(vel, s.vel.data(), s.vel.size() * 4);
    if (species) std::memcpy(species, s.species.data(), s.species.size() * 4);
}
void oracle_engine_set_state(void* h, const int64_t* pos, const int32_t* vel, const uint32_t* species) {
    State& s = ((Engine*)h)->state();
    std::memcpy(s.pos.data(), pos, s.pos.size() * 8);
    std::memcpy(s.vel.data(), vel, s.vel.size() * 4);
    std::memcpy(s.species.data(), species, s.species.size() * 4);
}
uint64_t oracle_engine_hash(void* h) { return ((Engine*)h)->state().hash(); }
void oracle_engine_ledger(void* h, double* energy, int64_t* energy_fixed, uint64_t* hits, uint32_t* clock) {
    Engine* e = (Engine*)h;
    const Ledger& l = e->f32 ? e->f32->ledger : e->f64->ledger;
    *energy = l.energy[LEDGER_BATH];
    *energy_fixed = l.bath_energy_fixed;
    *hits = l.hits[LEDGER_BATH];
    *clock = e->f32 ? e->f32->clock : e->f64->clock;
}
void oracle_engine_wall_ledger(void* h, double* energy, double* impulse, uint64_t* hits) {
    Engine* e = (Engine*)h;
    const Ledger& l = e->f32 ? e->f32->ledger : e->f64->ledger;
    for (int w = 0; w < LEDGER_SLOTS; w++) energy[w] = l.energy[w], impulse[w] = l.impulse[w], hits[w] = l.hits[w];
}
// System::with_bonds: ntypes bond types (fene 1 or harmonic 0, k, r0) and nbonds bonds
// (id a, id b, type), three words each.
void oracle_engine_set_bonds(void* h, const uint32_t* fene, const double* k, const double* r0, uint32_t ntypes, const uint32_t* bonds,
                             uint64_t nbonds) {
    std::vector<BondType> t(ntypes);
    for (uint32_t q = 0; q < ntypes; q++) t[q] = {fene[q] != 0, k[q], r0[q]};
    std::vector<std::array<uint32_t, 3>> b(nbonds);
    for (uint64_t q = 0; q < nbonds; q++) b[q] = {bonds[3 * q], bonds[3 * q + 1], bonds[3 * q + 2]};
    Engine* e = (Engine*)h;
    if (e->f32) e->f32->set_bonds(t, b);
    else e->f64->set_bonds(t, b);
}
// System::with_piston (system.rs:274-282): drive 0 none, 1 a set speed (sigma/tau), 2 free
// (mass, external force in eps/sigma); 0 on success, -1 for a system or piston it refuses.
int oracle_engine_set_piston(void* h, int drive, double speed, double mass, double force, double start, double min) {
    Engine* e = (Engine*)h;
    const bool ok = e->f32 ? e->f32->set_piston(drive, speed, mass, force, start, min) : e->f64->set_piston(drive, speed, mass, force, start, min);
    return ok ? 0 : -1;
}
// GpuEngine::set_piston_speed (md/src/engine.rs:936-939): the piston's velocity as a step
// displacement.
void oracle_engine_set_piston_speed(void* h, double speed) {
    Engine* e = (Engine*)h;
    if (e->f32) e->f32->piston_v = e->f32->sys.to_step_displacement(speed);
    else e->f64->piston_v = e->f64->sys.to_step_displacement(speed);
}
// The piston's height (position units), velocity (per step), the gas's work on it (eps) and
// the gas's force on it in the last force evaluation (eps/sigma).
void oracle_engine_piston(void* h, int64_t* w, int32_t* v, double* work, double* force) {
    Engine* e = (Engine*)h;
    if (e->f32) {
        *w = e->f32->piston_w, *v = e->f32->piston_v, *work = e->f32->piston_work, *force = e->f32->piston_force;
    } else {
        *w = e->f64->piston_w, *v = e->f64->piston_v, *work = e->f64->piston_work, *force = e->f64->piston_force;
    }
}
// The compartment ledger in integers: per_wall, then (energy, impulse, hits) per slot and
// compartment at [w per_wall + c] (arrays of at least LEDGER_SLOTS x per_wall; NULL: the count only).
uint32_t oracle_engine_compartment_ledger(void* h, int64_t* energy, int64_t* impulse, uint64_t* hits) {
    Engine* e = (Engine*)h;
    auto take = [&](auto* g) {
        if (energy)
            for (size_t q = 0; q < g->comp_hits.size(); q++) {
                energy[q] = g->comp_energy_fixed[q];
                impulse[q] = g->comp_impulse_fixed[q];
                hits[q] = g->comp_hits[q];
            }
        return g->per_wall;
    };
    return e->f32 ? take(e->f32.get()) : take(e->f64.get());
}
void oracle_engine_wall_ledger_fixed(void* h, int64_t* energy, int64_t* impulse) {
    const Ledger& l = ((Engine*)h)->f32 ? ((Engine*)h)->f32->ledger : ((Engine*)h)->f64->ledger;
    for (int w = 0; w < LEDGER_SLOTS; w++) {
        energy[w] = w == LEDGER_BATH ? l.bath_energy_fixed : l.energy_fixed[w];
        impulse[w] = l.impulse_fixed[w];
    }
}
void oracle_engine_set_system(void* h, const gbmd_system* csys) {
    Engine* e = (Engine*)h;
    System sys = System::from_c(*csys);
    if (e->f32) e->f32->set_system(sys);
    else e->f64->set_system(sys);
}
int64_t oracle_engine_steps(void* h) {
    Engine* e = (Engine*)h;
    return e->f32 ? e->f32->steps : e->f64->steps;
}
void oracle_engine_energy(void* h, double* ke, double* pe) {
    Engine* e = (Engine*)h;
    Energy en = e->f32 ? e->f32->energy() : e->f64->energy();
    *ke = en.kinetic;
    *pe = en.potential;
}
uint64_t oracle_state_hash(uint32_t dim, const int64_t* pos, const int32_t* vel, const uint32_t* species, uint64_t n) {
    return make_state((int)dim, pos, vel, species, n).hash();
}

void* oracle_float_create(const gbmd_system* csys, const int64_t* pos, const int32_t* vel, const uint32_t* species, uint64_t n) {
    System sys = System::from_c(*csys);
    return new FloatEngine(sys, make_state(2, pos, vel, species, n));
}
void oracle_float_destroy(void* h) { delete (FloatEngine*)h; }
void oracle_float_step(void* h, uint64_t steps) { ((FloatEngine*)h)->step(steps); }
void oracle_float_positions(void* h, double* out) {
    auto* e = (FloatEngine*)h;
    std::memcpy(out, e->pos.data(), e->pos.size() * 8);
}
void oracle_float_energy(void* h, double* ke, double* pe) {
    Energy en = ((FloatEngine*)h)->energy();
    *ke = en.kinetic;
    *pe = en.potential;
}

// ---- instruments
void oracle_pair_sums(const gbmd_system* csys, const int64_t* pos, const uint32_t* species, uint64_t n, double* pe, double* virial) {
    System sys = System::from_c(*csys);
    PairSums ps = pair_sums_f32(sys, make_state_pos(sys.dim, pos, species, n));
    *pe = ps.potential;
    *virial = ps.virial;
}
void oracle_rdf(const gbmd_system* csys, const int64_t* pos, uint64_t n, uint32_t bins, double rmax, uint64_t* out) {
    System sys = System::from_c(*csys);
    auto h = rdf_counts(sys, make_state_pos(sys.dim, pos, nullptr, n), bins, rmax);
    std::memcpy(out, h.data(), bins * 8);
}
void oracle_profile(const gbmd_system* csys, const int64_t* pos, uint64_t n, uint32_t bins, uint32_t axis, uint64_t* out) {
    System sys = System::from_c(*csys);
    auto h = density_profile(sys, make_state_pos(sys.dim, pos, nullptr, n), bins, (int)axis);
    std::memcpy(out, h.data(), bins * 8);
}
void oracle_fixed_speed(const gbmd_system* csys, const uint32_t* species, uint64_t n, double t, uint64_t seed, int32_t* vel) {
    System sys = System::from_c(*csys);
    auto v = fixed_speed(sys, std::vector<uint32_t>(species, species + n), t, seed);
    std::memcpy(vel, v.data(), v.size() * 4);
}
void oracle_barometric(const gbmd_system* csys, const uint32_t* species, uint64_t n, double t, double min_sep, double margin, uint64_t seed,
                       int64_t* pos) {
    System sys = System::from_c(*csys);
    auto p = barometric_positions(sys, std::vector<uint32_t>(species, species + n), t, min_sep, margin, seed);
    std::memcpy(pos, p.data(), p.size() * 8);
}
void oracle_mark_disc(const gbmd_system* csys, const int64_t* pos, uint32_t* species, uint64_t n, double cx, double cy, double radius,
                      uint32_t mark) {
    System sys = System::from_c(*csys);
    State s = make_state_pos(sys.dim, pos, species, n);
    const double c[2] = {cx, cy};
    mark_disc(sys, s, c, radius, mark);
    std::memcpy(species, s.species.data(), n * 4);
}
void oracle_observer_grid(const gbmd_system* csys, const int64_t* pos, const uint32_t* species, uint64_t n, uint32_t gx, uint32_t gy,
                          uint32_t marked, uint32_t* out) {
    System sys = System::from_c(*csys);
    auto h = observer_grid(sys, make_state_pos(sys.dim, pos, species, n), gx, gy, marked);
    std::memcpy(out, h.data(), h.size() * 4);
}

// ---- all-integer tables (md-core table.rs)
int oracle_int_kick(const gbmd_system* csys, uint32_t sa, uint32_t sb, const int64_t* d, int32_t* out) {
    System sys = System::from_c(*csys);
    IntTables t(sys);
    return t.kick(sa, sb, d, sys.dim, out) ? 1 : 0;
}

} // extern "C"
