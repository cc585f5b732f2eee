// The single-system engine behind the C ABI of include/gbmd.h: the GB300 counterpart of
// md::GpuEngine / md::GpuEngine3 (crates/md/src/engine.rs:598-1098, engine3.rs:334-648).
//
// One CUDA stream per engine. A step is: [if the rebuild flag is set: cell keys -> stable radix
// sort -> gather into cell order with the cell starts -> Verlet-list build] -> fused LJ force +
// leapfrog + displacement trigger. Steps are captured into CUDA graphs (blocks of
// `block_steps`), and the rebuild runs inside a conditional graph node whose condition a
// one-thread kernel reads from the device flag, so the decision never returns to the host (the
// reference's indirect-dispatch gate, gpu-prims prims.rs:250-283 / gate.wgsl:13-24). Small
// systems run a block as a persistent step loop instead (setup_step_loop, capture_loop_block):
// cooperative launches that step until the trigger fires, in a WHILE node with the rebuild in a
// nested IF.
#include <algorithm>
#include <array>
#include <cstddef>
#include <initializer_list>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "engine.cuh"
#include "kernels.cuh"
#include "half.cuh"
#include "sort.cuh"

namespace gbmd {

// ------------------------------------------------------------------ status + accounting
static thread_local std::string t_error;
void set_error(const std::string& msg) { t_error = msg; }
int fail(int code, const std::string& msg) {
    t_error = msg;
    return code;
}
static std::atomic<uint64_t> g_launches{0};
void note_launch(uint64_t k) { g_launches += k; }
uint64_t launch_total() { return g_launches.load(); }
// Engines alive in this process. The persistent step loop holds the whole grid of a cooperative
// launch for many steps; with several engines sharing the GPU their per-step graphs interleave
// better (1024 concurrent 2D engines: 3.20 x 10^9 atom-steps/s with per-step graphs, 2.16 with
// loops), so the loop runs only while its engine is the only one.
static std::atomic<int> g_live_engines{0};

static double to_f64h(int64_t x) { return (double)x * (1.0 / 4294967296.0); }

int validate_system(const gbmd_system& sys, uint32_t n) {
    if (sys.dim != 2 && sys.dim != 3) return fail(GBMD_E_INVALID, "dim must be 2 or 3");
    if (sys.nspecies < 1 || sys.nspecies > GBMD_MAX_SPECIES) return fail(GBMD_E_INVALID, "species must number 1 to 4");
    for (uint32_t a = 0; a < sys.dim; a++) {
        if ((sys.periodic >> a) & 1u) continue;
        for (int side = 0; side < 2; side++) {
            const uint32_t k = sys.wall_kind[a][side];
            if (k != GBMD_WALL_HARD && k != GBMD_WALL_SOFT && k != GBMD_WALL_THERMAL)
                return fail(GBMD_E_INVALID, "a non-periodic axis needs a wall (hard, soft or thermal) on each side");
            if (k == GBMD_WALL_THERMAL && !(sys.wall_t[a][side] >= 0.0 && sys.wall_t[a][side] < INFINITY))
                return fail(GBMD_E_INVALID, "a thermal wall needs a finite temperature >= 0");
        }
    }
    if (sys.membrane) {
        if (sys.dim != 2) return fail(GBMD_E_UNSUPPORTED, "membranes are two-dimensional (md_core::Membrane)");
        if (sys.membrane_axis >= 2 || ((sys.periodic >> sys.membrane_axis) & 1u))
            return fail(GBMD_E_INVALID, "a membrane lies across a walled axis (system.rs:259-265)");
        if (sys.membrane_pore_shift > 62) return fail(GBMD_E_INVALID, "bad membrane pore spacing");
    }
    if (sys.compartments[0] || sys.compartments[1]) {
        if (sys.dim != 2) return fail(GBMD_E_UNSUPPORTED, "compartments are two-dimensional (System::with_compartments)");
        for (uint32_t a = 0; a < 2; a++)
            if (sys.compartments[a] && (((sys.periodic >> a) & 1u) || sys.compartments[a] > 62))
                return fail(GBMD_E_INVALID, "compartments split a walled axis (system.rs:233-241)");
    }
    for (uint32_t a = 0; a < sys.dim; a++)
        if (sys.box_len[a] <= 0) return fail(GBMD_E_INVALID, "box lengths must be positive");
    for (uint32_t k = 0; k < sys.nspecies * sys.nspecies; k++) {
        const gbmd_pair& p = sys.pairs[k];
        if (!(p.rc < 7.9)) return fail(GBMD_E_INVALID, "cutoff must be below 8 sigma"); // system.rs:190-194
    }
    for (uint32_t s = 0; s < sys.nspecies; s++)
        if (!(sys.masses[s] > 0.0)) return fail(GBMD_E_INVALID, "masses must be positive");
    if (!(sys.dt > 0.0)) return fail(GBMD_E_INVALID, "dt must be positive");
    if (sys.bath) {
        if (!(sys.bath_t >= 0.0 && sys.bath_t < INFINITY) || !(sys.bath_rate >= 0.0 && sys.bath_rate < INFINITY))
            return fail(GBMD_E_INVALID, "the heat bath needs a finite temperature and rate, both >= 0");
        if (sys.bath_axis >= sys.dim || !(std::fabs(sys.bath_drift) < INFINITY)) return fail(GBMD_E_INVALID, "bad heat bath axis or drift");
    }
    (void)n;
    return GBMD_OK;
}

// ------------------------------------------------------------------ host-side System maths
double rc_max(const gbmd_system& s) {
    double r = 0.0;
    for (uint32_t k = 0; k < s.nspecies * s.nspecies; k++) r = std::max(r, s.pairs[k].rc);
    return r;
}
// System::cells_for (system.rs:438-444 / three.rs:151-157)
int cells_for(const gbmd_system& s, double r, uint32_t* c) {
    double bmax = 0.0;
    for (uint32_t a = 0; a < s.dim; a++) bmax = std::max(bmax, to_f64h(s.box_len[a]));
    double margin = 1e-3 + 1e-6 * bmax;
    c[2] = 1;
    for (uint32_t a = 0; a < s.dim; a++) {
        double v = std::floor(to_f64h(s.box_len[a]) / (r + margin));
        c[a] = v >= 4294967295.0 ? UINT32_MAX : (v > 0 ? (uint32_t)v : 0);
        if (c[a] < 3) return fail(GBMD_E_INVALID, "box too small for the cell radius (fewer than 3 cells on an axis)");
    }
    return GBMD_OK;
}
// Pair::shift (pair.rs:28-34) with Rust powi(6) = x^2 * (x^2)^2.
static double pair_shift(const gbmd_pair& p) {
    if (p.eps == 0.0 || p.rc == 0.0) return 0.0;
    double x = p.sigma / p.rc;
    double x2 = x * x;
    double s6 = x2 * (x2 * x2);
    return 4.0 * p.eps * s6 * (s6 - 1.0);
}
static float scale2(float v, int e) { return std::ldexp(v, e); }

// Rust's f64::powi: square-and-multiply from the low bit (the order sets the rounding).
static double powi_rs(double x, int n) {
    double res = 1.0, sq = x;
    bool have = false;
    while (n) {
        if (n & 1) {
            res = have ? res * sq : sq;
            have = true;
        }
        n >>= 1;
        if (n) sq = sq * sq;
    }
    return have ? res : 1.0;
}
static int64_t sat_i64_host(double x) {
    if (x != x) return 0;
    if (x >= 9223372036854775807.0) return INT64_MAX;
    if (x <= -9223372036854775808.0) return INT64_MIN;
    return (int64_t)x;
}
static int32_t sat_i32_host(double x) {
    if (x != x) return 0;
    if (x >= 2147483647.0) return INT32_MAX;
    if (x <= -2147483648.0) return INT32_MIN;
    return (int32_t)x;
}
static uint32_t sat_u32_host(double x) {
    if (!(x > 0.0)) return 0;
    if (x >= 4294967295.0) return UINT32_MAX;
    return (uint32_t)x;
}
// IntTables::new (crates/md-core/src/table.rs:45-71): per pair type, the kick coefficient
// 4 c f_over_r(r2) (f_over_r without its cutoff, pair.rs:45-51) rounded half away from zero at
// r2 = k 2^12 / 2^24 sigma^2 (k = 0 .. len - 1, r2 at least 0.36), zero beyond rc^2 + 2 steps.
static void int_tables(const gbmd_system& s, std::vector<int32_t>& data, uint32_t& len, uint32_t* irc2, std::vector<double>& pair4) {
    const uint32_t ns = s.nspecies;
    const double rcm = rc_max(s), rc2_max = rcm * rcm;
    len = (uint32_t)(((uint64_t)(rc2_max * 16777216.0) >> 12) + 2);
    data.assign((size_t)ns * ns * len, 0);
    pair4.assign((size_t)ns * ns * 4, 0.0);
    for (uint32_t a = 0; a < ns; a++) {
        const double c = ((s.pinned >> a) & 1u) ? 0.0 : s.dt * s.dt / s.masses[a] * 4294967296.0;
        for (uint32_t b = 0; b < ns; b++) {
            const gbmd_pair& p = s.pairs[a * ns + b];
            const uint32_t q = a * ns + b;
            irc2[q] = sat_u32_host(p.rc * p.rc * 16777216.0);
            pair4[4 * q] = p.eps;
            pair4[4 * q + 1] = p.sigma;
            pair4[4 * q + 2] = p.rc;
            pair4[4 * q + 3] = pair_shift(p);
            for (uint32_t k = 0; k < len; k++) {
                double r2 = (double)((uint64_t)k * 4096ull) / 16777216.0;
                r2 = std::max(r2, 0.36);
                double t = 0.0;
                if (r2 < p.rc * p.rc + 2.0 * 4096.0 / 16777216.0) {
                    const double s6 = powi_rs(p.sigma * p.sigma / r2, 3);
                    t = 24.0 * p.eps * s6 * (2.0 * s6 - 1.0) / r2 * c * 4.0;
                }
                double rt = std::round(t);
                rt = std::min(std::max(rt, -2147483648.0), 2147483647.0);
                data[(size_t)q * len + k] = sat_i32_host(rt);
            }
        }
    }
}

// Lower end of the scaled r2 range in which the pair chain uses rcp_cr / div_cr: 2^50 (r of
// 1/8 sigma) when, over [2^50, rc2s), t = c6 s6 (2 s6 - 1) stays below 2^100 in magnitude and its
// non-zero values above 2^-60 (so t / r2 is a normal f32), else +inf (library division only).
// Non-zero |2 s6 - 1| is at least 2^-24 (an f32 difference near 1), so |t| >= c6 s6min 2^-25.
float fast_pair_lo(const PairC& c) {
    const float lo = 0x1p50f;
    if (!(c.eps4 > 0.0f) || !(c.sigma2s > 0.0f) || !(c.rc2s > lo) || !(c.rc2s <= 0x1p62f)) return INFINITY;
    double s2max = (double)c.sigma2s / (double)lo, s2min = (double)c.sigma2s / (double)c.rc2s;
    double s6max = s2max * s2max * s2max * 1.01, s6min = s2min * s2min * s2min * 0.99;
    double tmax = (double)c.c6 * s6max * (2.0 * s6max + 1.0);
    double tmin = (double)c.c6 * std::min(s6min, 0.5) * 0x1p-25;
    if (!(tmax < 0x1p100) || !(tmin > 0x1p-60)) return INFINITY;
    return lo;
}

// System::to_step_displacement (system.rs:427-429): (v dt 2^32).round() as i32.
int32_t to_step_displacement(const gbmd_system& s, double v) { return sat_i32_host(std::round(v * s.dt * 4294967296.0)); }
void fill_params(Params& P, const gbmd_system& s, uint32_t n, double skin, uint32_t cap, const uint32_t* nc) {
    std::memset(&P, 0, sizeof(P));
    P.n = n;
    P.dim = s.dim;
    P.ns = s.nspecies;
    P.cap = cap;
    P.periodic = (s.periodic | (s.dim == 2 ? 4u : 0u)) & 7u;
    for (uint32_t a = 0; a < 3; a++) {
        P.box[a] = a < s.dim ? s.box_len[a] : 1;
        // (a walled axis: no separation reaches half, so min_image is the plain difference)
        P.half[a] = ((P.periodic >> a) & 1u) ? P.box[a] / 2 : INT64_MAX / 4;
        P.box_f[a] = to_f64h(P.box[a]);
        P.nc[a] = a < s.dim ? nc[a] : 1;
        if (a < s.dim && !((P.periodic >> a) & 1u)) {
            P.walls = 1;
            for (int side = 0; side < 2; side++) {
                P.wall_kind[a][side] = s.wall_kind[a][side];
                P.wall_t[a][side] = s.wall_t[a][side];
            }
        }
    }
    if (s.dim == 2) {
        P.membrane = s.membrane ? 1u : 0u;
        P.membrane_axis = s.membrane_axis;
        P.membrane_blocks = s.membrane_blocks;
        P.membrane_pore_shift = s.membrane_pore_shift;
        P.membrane_position = s.membrane_position;
        P.membrane_pore_width = s.membrane_pore_width;
        for (int a = 0; a < 2; a++) P.comp_shift[a] = s.compartments[a];
        P.comp_filter = (s.compartments[0] || s.compartments[1]) && !s.compartments_diathermal ? 1u : 0u;
    }
    P.wall_key[0] = (uint32_t)s.seed;
    P.wall_key[1] = (uint32_t)(s.seed >> 32) ^ 0x57414c4cu; // STREAM_WALL (walls.rs:86)
    P.ncell = P.nc[0] * P.nc[1] * P.nc[2];
    for (uint32_t sp = 0; sp < GBMD_MAX_SPECIES; sp++) {
        double kc = 0.0;
        if (sp < s.nspecies && !((s.pinned >> sp) & 1u)) kc = s.dt * s.dt / s.masses[sp] * 4294967296.0; // kick_coeff
        P.kick_cs[sp] = scale2((float)kc, 28);
        P.masses[sp] = sp < s.nspecies ? s.masses[sp] : 1.0;
    }
    for (uint32_t a = 0; a < 3; a++) {
        double g = a < s.dim ? s.gravity[a] : 0.0;
        P.grav_f[a] = g;
        double v = std::round(g * s.dt * s.dt * 4294967296.0); // System::gravity_kick
        P.gravity[a] = v != v ? 0 : (v >= 2147483647.0 ? INT32_MAX : (v <= -2147483648.0 ? INT32_MIN : (int32_t)v));
    }
    P.pinned = s.pinned;
    P.one = 1;
    double hs = 0.5 * skin * (1.0 - 1e-3);
    P.half_skin2s = scale2((float)(hs * hs), 56);
    // The trigger's f32 value for a displacement d is at most (|d| / 16)^2 (1 + 2^-21) (three
    // roundings of 2^-24), and |d| is at most the path U: U below 16 sqrt(half_skin2s) (1 - 2^-20)
    // cannot fire it.
    {
        const double u = 16.0 * std::sqrt((double)P.half_skin2s) * (1.0 - 0x1p-20);
        P.ub_thr = (s.dim == 2 && skin > 0.0 && u >= 1.0) ? (uint32_t)std::min(std::floor(u), 4294967294.0) : 0u;
    }
    P.dt = s.dt;
    for (uint32_t a = 0; a < s.nspecies; a++)
        for (uint32_t b = 0; b < s.nspecies; b++) {
            const gbmd_pair& p = s.pairs[a * s.nspecies + b];
            PairC& c = P.pc[a * s.nspecies + b];
            float rc2 = (float)(p.rc * p.rc), eps4 = (float)(4.0 * p.eps), sigma2 = (float)(p.sigma * p.sigma);
            c.rc2s = scale2(rc2, 56);
            c.sigma2s = scale2(sigma2, 56);
            c.eps4 = eps4;
            c.c6 = 6.0f * eps4;
            c.shift = (float)pair_shift(p);
            double lr = (p.rc + skin) * (1.0 + 1e-4);
            c.list2s = scale2((float)(lr * lr), 56);
            c.list2lo = (float)(lr * lr * (1.0 - 1e-4));
            c.list2hi = (float)(lr * lr * (1.0 + 1e-4));
            c.fast_lo = fast_pair_lo(c);
        }
    // Listed pairs: within the list radius at the build; each particle has moved less than half
    // the skin before the trigger fires and at most 0.5 sigma per axis (an i32 displacement) in
    // the step after it, so |d| < r_list + skin + 2 sqrt(3) 0.5 sigma < r_list + skin + 2 sigma.
    double r_list = (rc_max(s) + skin) * (1.0 + 1e-4);
    P.reach = (int64_t)std::ceil((r_list + skin + 2.0) * 4294967296.0);
    set_cells(P, P.nc, s.dim);
    if (s.bath) {
        // walls::andersen / three::andersen: the threshold rate dt, sqrt(t / m) per species, the
        // thermostat key (walls.rs:110, STREAM_THERMO) and the fan's drift in integer units
        P.bath = 1;
        P.bath_species = s.bath_species;
        P.bath_axis = s.dim == 2 ? s.bath_axis : 0;
        P.bath_drift = s.dim == 2 ? to_step_displacement(s, s.bath_drift) : 0;
        P.bath_region[0] = s.dim == 2 ? s.bath_region[0] : INT64_MIN;
        P.bath_region[1] = s.dim == 2 ? s.bath_region[1] : INT64_MAX;
        P.bath_rate_dt = s.bath_rate * s.dt;
        for (uint32_t sp = 0; sp < s.nspecies; sp++) P.bath_sd[sp] = std::sqrt(s.bath_t / s.masses[sp]);
        P.bath_key[0] = (uint32_t)s.seed;
        P.bath_key[1] = (uint32_t)(s.seed >> 32) ^ 0x5448524du;
    }
}

// Cell grid of a parameter block: counts, the f32 cell-index helpers and whether candidates of
// adjacent cells are certainly within 8 sigma per axis.
void set_cells(Params& P, const uint32_t* nc, uint32_t dim) {
    for (uint32_t a = 0; a < 3; a++) P.nc[a] = a < dim ? nc[a] : 1;
    P.ncell = P.nc[0] * P.nc[1] * P.nc[2];
    P.key_shift = 0;
    P.sub_scale = 0.0f;
    P.sub_delta = 0;
    double side = 0.0;
    for (uint32_t a = 0; a < dim; a++) side = std::max(side, P.box_f[a] / (double)P.nc[a]);
    P.sep_unchecked = 2.0 * side < 7.99 ? 1u : 0u;
    for (uint32_t a = 0; a < 3; a++) {
        P.cell_w[a] = P.box[a] / (int64_t)P.nc[a];
        double sc = (double)P.nc[a] / (P.box_f[a] * 4294967296.0);
        P.cell_scale_f[a] = (float)sc;
        // |f32 product - exact| <= 3 2^-24 (x n / L) < 2^-22 n (x < L); twice that as margin
        P.cell_delta[a] = (float)std::min(0.5, std::ldexp((double)P.nc[a], -21));
    }
}
int key_bits(uint32_t ncell) {
    int b = 0;
    while (b < 32 && (ncell - 1) >> b) b++;
    return std::max(b, 1);
}

// List builds: each cell's particles sorted by 2^shift slabs of their last coordinate, so that a
// particle scans only the slabs of the cells one layer up (down) that can hold a neighbour: those
// at or below (above) its own slab, 3D: 9 (2 + 2^-shift) cells instead of 27 per lane. The lanes
// of one warp cover every slab of a cell, so the warp's walk shrinks only when a particle has
// several lanes: used for multi-lane builds (small systems) only, where with one lane per
// particle the lanes' different slab ranges only add divergence. The shift is the largest that
// adds no radix pass to the sort.
static void set_sub_buckets(Params& P, uint32_t dim, double r_list) {
    const uint32_t a = dim - 1;
    const int64_t w = P.cell_w[a];
    if (w <= 256 || w >= ((int64_t)1 << 38)) return; // sub_bucket converts (z_rel >> 8) to i32
    const int bits = key_bits(P.ncell);
    int shift = 3;
    while (shift > 0 && (bits + shift > 31 || radix_passes(bits + shift) > radix_passes(bits))) shift--;
    if (shift == 0) return;
    P.key_shift = (uint32_t)shift;
    P.sub_scale = (float)((double)(1u << shift) / (double)(w >> 8));
    // A pair the exact list test accepts has |d| < r_list (1 + 2^-21) + 16 on every axis (the f32
    // roundings of list2s, r2 and the separation); with the cell side w, a neighbour in the next
    // layer up then sits at most reach - w above the particle's own offset in its cell.
    const double reach = r_list * (1.0 + 0x1p-20) * 4294967296.0 + 64.0;
    P.sub_delta = reach > (double)w ? (int64_t)std::ceil(reach - (double)w) : 0;
}
static uint32_t blocks_for(uint64_t n, uint32_t t) { return (uint32_t)((n + t - 1) / t); }

} // namespace gbmd

using namespace gbmd;

// ------------------------------------------------------------------ the engine
struct gbmd_engine {
    gbmd_system sys{};
    gbmd_options opt{};
    uint32_t n = 0;
    int D = 2;
    bool verlet = true;
    bool multi = false;
    double skin = 0.0;
    Params P{};     // force/list parameters (cells of rc + skin)
    int bits = 1;   // significant bits of the cell keys
    cudaStream_t st = nullptr;
    cudaStream_t st_body = nullptr; // capture stream of conditional bodies
    cudaStream_t st_body2 = nullptr; // and of conditional bodies nested in them
    size_t rec = 16; // bytes per position record

    void* pos[2] = {nullptr, nullptr};
    void* pos_scr = nullptr;
    void* ref_pos = nullptr;
    int32_t *vel = nullptr, *vel_scr = nullptr, *kicks = nullptr;
    uint32_t *species = nullptr, *species_scr = nullptr, *ids = nullptr, *ids_scr = nullptr;
    uint32_t *keys[2] = {nullptr, nullptr}, *vals[2] = {nullptr, nullptr};
    uint32_t *hist = nullptr, *scan_tmp = nullptr, *start = nullptr;
    uint32_t *nbr = nullptr, *nbr_count = nullptr;
    float4* relf = nullptr;  // cell-relative f32 coordinates of the sorted scratch state
    uint4* qpos[2] = {nullptr, nullptr}; // quotient records of the positions (ping-pong)
    uint32_t* ctl = nullptr; // [0] rebuild, [1] overflow, [2] rebuilds; [CTL_CLOCK] the bath's step clock
    unsigned long long* ledger = nullptr; // per ledger slot: energy given (2^-24 epsilon), hits, impulse (2^-24)
    double* partial = nullptr;
    void* staging = nullptr;  // id-ordered I/O staging (n * D int64)
    int32_t* staging_v = nullptr;
    uint32_t* staging_s = nullptr;
    int sorted = 0; // which keys/vals buffer holds the sorted result

    int cur = 0;
    int64_t steps = 0;
    uint32_t clock = 0;
    uint32_t block_steps = 64;
    // graphs per [parity][kind]: 0 one step, 1 a block of block_steps, 2 one step + thermostat,
    // 3 the conditional list rebuild alone (frames and kicks between steps)
    // 4 a block of block_steps through the persistent step loop (small systems)
    cudaGraphExec_t exec[2][5] = {{nullptr, nullptr, nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr, nullptr, nullptr}};
    uint64_t exec_launches[2][5] = {{0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}};
    uint32_t loop_lanes = 0;  // lanes per particle of the persistent step loop (0: not used)
    uint32_t loop_blocks = 0; // its grid
    uint32_t loop_iters = 0;  // its launches so far
    bool live = false;        // counted in g_live_engines
    // velocity-rescale thermostat (every `rescale_every` steps)
    uint32_t* mrank = nullptr;          // rank of each id among the moving particles
    unsigned long long* tpart = nullptr; // exact KE partials
    long long* vpart = nullptr;          // velocity-sum partials
    double* tfac = nullptr;              // factor + skip flag
    uint32_t thermo_nb = 1;
    uint32_t moving = 0;
    uint64_t tcount = 0;                 // steps since creation (thermostat phase)
    uint64_t body_launches = 0;
    uint64_t launches = 0;
    uint32_t last_rebuilds = 0;
    bool failed = false;
    bool half = false;       // half-shell lists (k_build_half / k_force_half / k_leap_half)
    uint32_t* bond_tab = nullptr; // bonds: per id 4 x (partner id, type), padded with UINT32_MAX
    std::vector<gbmd_bond_type> bond_types_h;        // the bond types and bonds as set (host copies:
    std::vector<std::array<uint32_t, 3>> bonds_h;     // add_bond / remove_bond edit them)
    uint32_t* slot_of = nullptr;  // bonds: the storage slot of each id
    PistonState* piston = nullptr; // the piston's moving state (2D)
    int32_t* acc = nullptr;  // half-shell kick accumulators, 3 x int32 per slot, zero between steps
    int32_t* itab = nullptr; // all-integer kick tables (GBMD_ARITH_INT)
    double* ipair = nullptr;
    // observation scratch, kept between frames (freeing it would synchronise the whole device)
    unsigned long long* obs_bins = nullptr;
    size_t obs_bins_cap = 0;
    uint32_t* obs_start = nullptr;
    size_t obs_start_cap = 0;
    // a frame in flight (gbmd_observe_begin .. gbmd_observe_end): results land in pinned memory
    double* obs_part_h = nullptr;
    size_t obs_part_cap = 0;
    unsigned long long* obs_bins_h = nullptr;
    size_t obs_bins_h_cap = 0;
    bool obs_pending = false;
    uint32_t obs_rdf_bins = 0, obs_profile_bins = 0, obs_nb = 0;
};

namespace {

template <int D> using Rec = PosRec<D>;

// Engine memory comes from the stream-ordered allocator on the engine's own stream, and goes back
// to it the same way: creating and destroying engines (a server does so per request) never
// synchronises the device with other engines' work. The device's default pool keeps what is
// freed for the next engine (release threshold raised once per device).
static void keep_pool_memory(int device) {
    static std::mutex mu;
    static bool done[256] = {false};
    std::lock_guard<std::mutex> lock(mu);
    if (device < 0 || device >= 256 || done[device]) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    done[device] = true;
}
int alloc(gbmd_engine* e, void** p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    cudaError_t r = cudaMallocAsync(p, bytes, e->st);
    if (r != cudaSuccess) return fail(r == cudaErrorMemoryAllocation ? GBMD_E_NOMEM : GBMD_E_CUDA, std::string("cudaMallocAsync: ") + cudaGetErrorString(r));
    return GBMD_OK;
}
template <typename T> int allocT(gbmd_engine* e, T** p, size_t count) { return alloc(e, (void**)p, count * sizeof(T)); }

// Pinned host memory for frames, from a process-wide pool that is never freed (freeing pinned
// memory synchronises the device): blocks of a power-of-two size, handed out and taken back.
static std::mutex g_pin_mu;
static std::map<size_t, std::vector<void*>> g_pin_free;
static size_t pin_class(size_t bytes) {
    size_t c = 4096;
    while (c < bytes) c <<= 1;
    return c;
}
static void* pinned_take(size_t cls) {
    {
        std::lock_guard<std::mutex> lock(g_pin_mu);
        auto it = g_pin_free.find(cls);
        if (it != g_pin_free.end() && !it->second.empty()) {
            void* p = it->second.back();
            it->second.pop_back();
            return p;
        }
    }
    void* p = nullptr;
    return cudaHostAlloc(&p, cls, cudaHostAllocDefault) == cudaSuccess ? p : nullptr;
}
static void pinned_give(void* p, size_t cls) {
    if (!p) return;
    std::lock_guard<std::mutex> lock(g_pin_mu);
    g_pin_free[cls].push_back(p);
}

void free_all(gbmd_engine* e) {
    if (e->live) {
        e->live = false;
        g_live_engines--;
    }
    for (int p = 0; p < 2; p++)
        for (int b = 0; b < 5; b++)
            if (e->exec[p][b]) cudaGraphExecDestroy(e->exec[p][b]);
    void* ptrs[] = {e->pos[0], e->pos[1], e->pos_scr, e->ref_pos, e->vel, e->vel_scr, e->kicks, e->species, e->species_scr, e->ids,
                    e->ids_scr, e->keys[0], e->keys[1], e->vals[0], e->vals[1], e->hist, e->scan_tmp, e->start, e->nbr,
                    e->nbr_count, e->ctl, e->partial, e->staging, e->staging_v, e->staging_s, e->mrank, e->tpart, e->vpart, e->tfac, e->relf, e->qpos[0], e->qpos[1],
                    e->obs_bins, e->obs_start, e->itab, e->ipair, e->ledger, e->acc, e->bond_tab, e->slot_of};
    for (void* p : ptrs)
        if (p) cudaFreeAsync(p, e->st);
    if (e->st) cudaStreamDestroy(e->st);
    if (e->st_body) cudaStreamDestroy(e->st_body);
    if (e->st_body2) cudaStreamDestroy(e->st_body2);
    pinned_give(e->obs_part_h, e->obs_part_cap);
    pinned_give(e->obs_bins_h, e->obs_bins_h_cap);
}

// ---- enqueue helpers (stream-ordered; also used under capture)
// keys + first histogram -> radix passes -> gather with the cell starts (n >= 1).
template <int D> void enqueue_bin(gbmd_engine* e, cudaStream_t s, const Params& P) {
    const uint32_t nkeys = P.ncell << P.key_shift; // cells x slabs (list builds) or cells
    const uint32_t tiles = blocks_for(e->n, RADIX_TILE);
    k_keys_hist<D><<<tiles, 256, 0, s>>>(P, (const Rec<D>*)e->pos[e->cur], e->keys[0], e->vals[0], e->hist, tiles);
    uint32_t sort_launches = 0;
    e->sorted = radix_sort_pairs(e->keys[0], e->vals[0], e->keys[1], e->vals[1], e->n, key_bits(nkeys), e->hist, e->scan_tmp, s, true,
                                 &sort_launches);
    k_gather<D><<<blocks_for(e->n, 256), 256, 0, s>>>(P, e->vals[e->sorted], e->keys[e->sorted], (const Rec<D>*)e->pos[e->cur], e->vel,
                                                       e->species, e->ids, (Rec<D>*)e->pos_scr, e->vel_scr, e->species_scr, e->ids_scr,
                                                       e->relf, e->start, nkeys);
    note_launch(2 + sort_launches);
}

// Lanes per particle of the list build: one for large systems, more below these counts, where a
// lane per particle would leave most of the GPU idle during its ~500-candidate walk.
static uint32_t build_lanes(uint32_t n) { return n < 24576 ? 8u : (n < 49152 ? 4u : (n < 98304 ? 2u : 1u)); }
static uint32_t list_build_lanes(const gbmd_engine* e) {
    const uint32_t o = (e->opt.flags >> 4) & 15u;
    return o ? o : build_lanes(e->n);
}

template <int D, bool MULTI> void enqueue_rebuild_t(gbmd_engine* e, cudaStream_t s, bool full) {
    enqueue_bin<D>(e, s, e->P);
    if constexpr (D == 3 && !MULTI) {
        if (e->half && !full) {
            k_build_half<<<blocks_for(e->n, 128), 128, 0, s>>>(e->P, (const Rec<3>*)e->pos_scr, e->vel_scr, e->species_scr, e->ids_scr,
                                                               e->keys[e->sorted], e->start, e->relf, (Rec<3>*)e->pos[e->cur], e->vel,
                                                               e->species, e->ids, (Rec<3>*)e->ref_pos, e->nbr, e->nbr_count, e->ctl,
                                                               e->qpos[e->cur]);
            note_launch();
            return;
        }
    }
#define GBMD_BUILD(SS)                                                                                                              \
    k_build_list<D, MULTI, SS><<<blocks_for((uint64_t)e->n * SS, 128), 128, 0, s>>>(                                               \
        e->P, (const Rec<D>*)e->pos_scr, e->vel_scr, e->species_scr, e->ids_scr, e->keys[e->sorted], e->start, e->relf,            \
        (Rec<D>*)e->pos[e->cur], e->vel, e->species, e->ids, (Rec<D>*)e->ref_pos, e->nbr, e->nbr_count, e->ctl, e->qpos[e->cur])
    switch (list_build_lanes(e)) {
    case 8: GBMD_BUILD(8); break;
    case 4: GBMD_BUILD(4); break;
    case 2: GBMD_BUILD(2); break;
    default: GBMD_BUILD(1); break;
    }
#undef GBMD_BUILD
    note_launch();
    if constexpr (D == 2) {
        if (e->P.comp_filter) {
            k_filter_compartments<<<blocks_for(e->n, 128), 128, 0, s>>>(e->P, (const Rec<2>*)e->pos[e->cur], e->nbr, e->nbr_count);
            note_launch();
        }
    }
}

__global__ void k_set_cond(cudaGraphConditionalHandle h, const uint32_t* ctl) { cudaGraphSetConditional(h, ctl[0] ? 1u : 0u); }

// The list the engine steps with (half-shell lists on a half engine), or with `full` a full list
// whatever the engine (the instruments and reversal walk full lists).
void enqueue_rebuild(gbmd_engine* e, cudaStream_t s, bool full = false) {
    if (e->D == 2) {
        if (e->multi) enqueue_rebuild_t<2, true>(e, s, full);
        else enqueue_rebuild_t<2, false>(e, s, full);
    } else {
        if (e->multi) enqueue_rebuild_t<3, true>(e, s, full);
        else enqueue_rebuild_t<3, false>(e, s, full);
    }
    if (e->verlet && e->P.bonds && e->D == 2) { // the slots of the ids, which only a list build moves
        k_slot_of<<<blocks_for(e->n, 256), 256, 0, s>>>(e->n, e->ids, e->slot_of);
        note_launch();
    }
}
__global__ void k_set_trigger(uint32_t* ctl) { ctl[0] = 1; }

// Below these particle counts the force kernel runs 8 (4, 2) lanes per particle.
constexpr uint32_t FORCE_SPLIT8_BELOW = 20000, FORCE_SPLIT4_BELOW = 65536, FORCE_SPLIT2_BELOW = 262144;
// Lanes per particle of the force step (single species, f32 chain): gbmd_options.flags bits 8-12
// when set (1, 2, 4, 8 or 16), else by size.
static uint32_t force_lanes(const gbmd_engine* e) {
    const uint32_t o = (e->opt.flags >> 8) & 31u;
    if (o == 1 || o == 2 || o == 4 || o == 8 || o == 16) return o;
    return e->n < FORCE_SPLIT8_BELOW ? 8u : (e->n < FORCE_SPLIT4_BELOW ? 4u : (e->n < FORCE_SPLIT2_BELOW ? 2u : 1u));
}
// Whether the force kernel takes the scenario's bonds, walls, piston and bath in its own epilogue
// (Verlet lists, f32 pairs, one lane per particle): one pass over the state instead of up to three.
static bool scenario_epilogue(const gbmd_engine* e) {
    if (!e->verlet || e->half || e->P.int_mode) return false;
    if (!(e->P.walls || (e->P.bonds && e->D == 2) || e->P.bath)) return false;
    return e->multi || force_lanes(e) == 1;
}
template <int D, bool MULTI, bool INT> void enqueue_force_a(gbmd_engine* e, cudaStream_t s, uint32_t threads) {
    if constexpr (D == 3 && !MULTI && !INT) {
        if (e->half) {
            const size_t smem = (size_t)e->P.win_cap * 12;
            const uint32_t rows = e->P.nc[1] * e->P.nc[2];
            if (e->P.pc[0].sigma2s == 0x1p56f)
                k_force_half<true><<<rows, HALF_THREADS, smem, s>>>(e->P, e->qpos[e->cur], e->nbr, e->nbr_count, e->start, e->acc);
            else
                k_force_half<false><<<rows, HALF_THREADS, smem, s>>>(e->P, e->qpos[e->cur], e->nbr, e->nbr_count, e->start, e->acc);
            k_leap_half<<<blocks_for(e->n, 256), 256, 0, s>>>(e->P, (const Rec<3>*)e->pos[e->cur], (Rec<3>*)e->pos[e->cur ^ 1],
                                                             e->qpos[e->cur ^ 1], e->vel, (int4*)e->acc, (const Rec<3>*)e->ref_pos, e->ctl);
            note_launch(2);
            e->cur ^= 1;
            return;
        }
    }
    if (e->verlet) {
        // sigma = 1 for every pair type (the common LJ case): compiled into the f32 chain
        bool sig1 = !INT;
        for (uint32_t k = 0; k < e->P.ns * e->P.ns; k++) sig1 = sig1 && e->P.pc[k].sigma2s == 0x1p56f;
        // small single-species systems: several lanes per particle (force_lanes)
        const uint32_t split = (!INT && !MULTI) ? force_lanes(e) : 1u;
        if (split > 1) {
            const uint32_t lanes = (uint32_t)(((uint64_t)e->n * split + 31) / 32 * 32);
#define GBMD_SPLIT(SS, SG)                                                                                                          \
    k_force_list<D, false, false, SG, SS><<<blocks_for(lanes, threads), threads, 0, s>>>(                                            \
        e->P, (const Rec<D>*)e->pos[e->cur], (Rec<D>*)e->pos[e->cur ^ 1], e->qpos[e->cur], e->qpos[e->cur ^ 1], e->vel, e->species, \
        e->nbr, e->nbr_count, (const Rec<D>*)e->ref_pos, e->ctl)
            if (split == 16) {
                if (sig1) GBMD_SPLIT(16, true);
                else GBMD_SPLIT(16, false);
            } else if (split == 8) {
                if (sig1) GBMD_SPLIT(8, true);
                else GBMD_SPLIT(8, false);
            } else if (split == 4) {
                if (sig1) GBMD_SPLIT(4, true);
                else GBMD_SPLIT(4, false);
            } else {
                if (sig1) GBMD_SPLIT(2, true);
                else GBMD_SPLIT(2, false);
            }
#undef GBMD_SPLIT
        } else if (!INT && scenario_epilogue(e)) {
            if (sig1 && !MULTI)
                k_force_list<D, MULTI, false, true, 1, true><<<blocks_for(e->n, threads), threads, 0, s>>>(
                    e->P, (const Rec<D>*)e->pos[e->cur], (Rec<D>*)e->pos[e->cur ^ 1], e->qpos[e->cur], e->qpos[e->cur ^ 1], e->vel,
                    e->species, e->nbr, e->nbr_count, (const Rec<D>*)e->ref_pos, e->ctl);
            else
                k_force_list<D, MULTI, false, false, 1, true><<<blocks_for(e->n, threads), threads, 0, s>>>(
                    e->P, (const Rec<D>*)e->pos[e->cur], (Rec<D>*)e->pos[e->cur ^ 1], e->qpos[e->cur], e->qpos[e->cur ^ 1], e->vel,
                    e->species, e->nbr, e->nbr_count, (const Rec<D>*)e->ref_pos, e->ctl);
        } else if (sig1)
            k_force_list<D, MULTI, INT, true><<<blocks_for(e->n, threads), threads, 0, s>>>(
                e->P, (const Rec<D>*)e->pos[e->cur], (Rec<D>*)e->pos[e->cur ^ 1], e->qpos[e->cur], e->qpos[e->cur ^ 1], e->vel,
                e->species, e->nbr, e->nbr_count, (const Rec<D>*)e->ref_pos, e->ctl);
        else
            k_force_list<D, MULTI, INT, false><<<blocks_for(e->n, threads), threads, 0, s>>>(
                e->P, (const Rec<D>*)e->pos[e->cur], (Rec<D>*)e->pos[e->cur ^ 1], e->qpos[e->cur], e->qpos[e->cur ^ 1], e->vel,
                e->species, e->nbr, e->nbr_count, (const Rec<D>*)e->ref_pos, e->ctl);
        note_launch();
        e->cur ^= 1;
    } else {
        enqueue_bin<D>(e, s, e->P);
        k_force_cells<D, MULTI, INT><<<blocks_for(e->n, threads), threads, 0, s>>>(e->P, (const Rec<D>*)e->pos_scr, e->vel_scr,
                                                                                 e->species_scr, e->ids_scr, e->keys[e->sorted], e->start,
                                                                                 (Rec<D>*)e->pos[e->cur], e->vel, e->species, e->ids);
        note_launch();
    }
}
template <int D, bool MULTI> void enqueue_force_t(gbmd_engine* e, cudaStream_t s, uint32_t threads) {
    if (e->P.int_mode) enqueue_force_a<D, MULTI, true>(e, s, threads);
    else enqueue_force_a<D, MULTI, false>(e, s, threads);
}
__global__ void k_clock_tick(uint32_t* ctl) { ctl[CTL_CLOCK] += 1u; }
__global__ void k_clock_set(uint32_t* ctl, uint32_t clock) { ctl[CTL_CLOCK] = clock; }

void enqueue_force(gbmd_engine* e, cudaStream_t s) {
    uint32_t threads = e->opt.threads ? e->opt.threads : 128;
    if (e->D == 2) {
        if (e->multi) enqueue_force_t<2, true>(e, s, threads);
        else enqueue_force_t<2, false>(e, s, threads);
    } else {
        if (e->multi) enqueue_force_t<3, true>(e, s, threads);
        else enqueue_force_t<3, false>(e, s, threads);
    }
    const bool epi = scenario_epilogue(e);
    if (epi) { // the force kernel took the bonds, walls, piston and bath: the piston moves, the clock
        if (e->P.walls || e->P.bath) {
            if (e->P.piston_drive) k_piston_tick<<<1, 1, 0, s>>>(e->P, e->ctl);
            else k_clock_tick<<<1, 1, 0, s>>>(e->ctl);
            note_launch();
        }
        return;
    }
    if (e->P.bonds && e->D == 2) { // the bonds' kicks from the step's start positions
        const uint32_t nb = blocks_for(e->n, 256);
        k_slot_of<<<nb, 256, 0, s>>>(e->n, e->ids, e->slot_of);
        if (e->verlet)
            k_bonds<2, true><<<nb, 256, 0, s>>>(e->P, (const Rec<2>*)e->pos[e->cur ^ 1], (Rec<2>*)e->pos[e->cur], e->qpos[e->cur], e->vel,
                                                e->species, e->ids, (const Rec<2>*)e->ref_pos, e->ctl);
        else
            k_bonds<2, false><<<nb, 256, 0, s>>>(e->P, (const Rec<2>*)e->pos_scr, (Rec<2>*)e->pos[e->cur], nullptr, e->vel, e->species,
                                                 e->ids, nullptr, e->ctl);
        note_launch(2);
    }
    if (e->P.walls) { // the soft walls' kicks, the bath, the mirror and collisions; then the clock
        const uint32_t nb = blocks_for(e->n, 256);
        unsigned long long* l = e->ledger;
        if (e->D == 2) {
            if (e->verlet) k_walls<2, true><<<nb, 256, 0, s>>>(e->P, (Rec<2>*)e->pos[e->cur], e->qpos[e->cur], e->vel, e->species, e->ids, (const Rec<2>*)e->ref_pos, e->ctl, l);
            else k_walls<2, false><<<nb, 256, 0, s>>>(e->P, (Rec<2>*)e->pos[e->cur], nullptr, e->vel, e->species, e->ids, nullptr, e->ctl, l);
        } else {
            if (e->verlet) k_walls<3, true><<<nb, 256, 0, s>>>(e->P, (Rec<3>*)e->pos[e->cur], e->qpos[e->cur], e->vel, e->species, e->ids, (const Rec<3>*)e->ref_pos, e->ctl, l);
            else k_walls<3, false><<<nb, 256, 0, s>>>(e->P, (Rec<3>*)e->pos[e->cur], nullptr, e->vel, e->species, e->ids, nullptr, e->ctl, l);
        }
        if (e->P.piston_drive) k_piston_tick<<<1, 1, 0, s>>>(e->P, e->ctl); // the piston moves, then the clock
        else k_clock_tick<<<1, 1, 0, s>>>(e->ctl);
        note_launch(2);
    } else if (e->P.bath) { // the Andersen bath on the moved state, then the step clock advances
        const uint32_t nb = blocks_for(e->n, 256);
        if (e->D == 2) {
            if (e->verlet) k_bath<2, true><<<nb, 256, 0, s>>>(e->P, (Rec<2>*)e->pos[e->cur], e->qpos[e->cur], e->vel, e->species, e->ids, (const Rec<2>*)e->ref_pos, e->ctl, e->ledger + 3 * (size_t)GBMD_LEDGER_BATH * e->P.ledger_per_wall);
            else k_bath<2, false><<<nb, 256, 0, s>>>(e->P, (Rec<2>*)e->pos[e->cur], nullptr, e->vel, e->species, e->ids, nullptr, e->ctl, e->ledger + 3 * (size_t)GBMD_LEDGER_BATH * e->P.ledger_per_wall);
        } else {
            if (e->verlet) k_bath<3, true><<<nb, 256, 0, s>>>(e->P, (Rec<3>*)e->pos[e->cur], e->qpos[e->cur], e->vel, e->species, e->ids, (const Rec<3>*)e->ref_pos, e->ctl, e->ledger + 3 * (size_t)GBMD_LEDGER_BATH * e->P.ledger_per_wall);
            else k_bath<3, false><<<nb, 256, 0, s>>>(e->P, (Rec<3>*)e->pos[e->cur], nullptr, e->vel, e->species, e->ids, nullptr, e->ctl, e->ledger + 3 * (size_t)GBMD_LEDGER_BATH * e->P.ledger_per_wall);
        }
        k_clock_tick<<<1, 1, 0, s>>>(e->ctl);
        note_launch(2);
    }
}

// The velocity-rescale thermostat: exact KE -> factor -> v <- round(v f) -> exact zero sum.
void enqueue_thermo(gbmd_engine* e, cudaStream_t s) {
    ThermoP T{};
    T.nblocks = e->thermo_nb;
    T.ns = e->sys.nspecies;
    for (uint32_t k = 0; k < GBMD_MAX_SPECIES; k++) T.masses[k] = k < e->sys.nspecies ? e->sys.masses[k] : 1.0;
    T.dt = e->sys.dt;
    T.dof = 0.5 * e->D * std::max((double)e->moving - 1.0, 1.0);
    T.t = e->opt.rescale_t;
    uint32_t nb = e->thermo_nb;
    if (e->D == 2) {
        k_ke_exact<2><<<nb, 256, 0, s>>>(e->n, e->vel, e->species, e->sys.pinned, e->tpart);
        k_thermo_factor<<<1, 256, 0, s>>>(T, e->tpart, e->tfac);
        k_rescale<2><<<nb, 256, 0, s>>>(e->n, e->vel, e->species, e->sys.pinned, e->tfac, e->vpart);
        k_vsum<<<1, 256, 0, s>>>(e->vpart, nb, e->vpart + 3 * (size_t)nb);
        k_zero_apply<2><<<blocks_for(e->n, 256), 256, 0, s>>>(e->n, e->vel, e->species, e->ids, e->mrank, e->sys.pinned, e->moving,
                                                               e->vpart + 3 * (size_t)nb, e->tfac);
    } else {
        k_ke_exact<3><<<nb, 256, 0, s>>>(e->n, e->vel, e->species, e->sys.pinned, e->tpart);
        k_thermo_factor<<<1, 256, 0, s>>>(T, e->tpart, e->tfac);
        k_rescale<3><<<nb, 256, 0, s>>>(e->n, e->vel, e->species, e->sys.pinned, e->tfac, e->vpart);
        k_vsum<<<1, 256, 0, s>>>(e->vpart, nb, e->vpart + 3 * (size_t)nb);
        k_zero_apply<3><<<blocks_for(e->n, 256), 256, 0, s>>>(e->n, e->vel, e->species, e->ids, e->mrank, e->sys.pinned, e->moving,
                                                               e->vpart + 3 * (size_t)nb, e->tfac);
    }
    note_launch(5);
}

// Ranks of the moving particles in id order (zero_velocity_sum's order) from id-ordered species.
int upload_ranks(gbmd_engine* e, const uint32_t* species) {
    std::vector<uint32_t> r(e->n, 0);
    uint32_t k = 0;
    for (uint32_t i = 0; i < e->n; i++)
        if (!((e->sys.pinned >> species[i]) & 1u)) r[i] = k++;
    e->moving = k;
    GBMD_CUDA_TRY(cudaMemcpyAsync(e->mrank, r.data(), (size_t)e->n * 4, cudaMemcpyHostToDevice, e->st));
    GBMD_CUDA_TRY(cudaStreamSynchronize(e->st));
    return GBMD_OK;
}

// ---- the persistent step loop (graph kind 4)
constexpr uint32_t CTL_WHILE_ITERS = 10; // WHILE iterations in the current block
constexpr uint32_t STEP_LOOP_BELOW = 98304; // particles: the loop is used below this
__global__ void k_loop_begin(uint32_t* ctl) {
    ctl[CTL_LOOP_DONE] = 0;
    ctl[CTL_WHILE_ITERS] = 0;
}
// Repeat the block's body while steps remain. Every iteration takes at least one step (the
// rebuild before it clears the trigger), so more than target + 1 iterations means something is
// wrong: stop then too, as after a barrier that ran out.
__global__ void k_set_while(cudaGraphConditionalHandle h, uint32_t* ctl, uint32_t target) {
    const uint32_t it = ctl[CTL_WHILE_ITERS] + 1u;
    ctl[CTL_WHILE_ITERS] = it;
    const bool more = ctl[CTL_LOOP_DONE] < target && ctl[CTL_LOOP_ERR] == 0u && it <= target + 1u;
    cudaGraphSetConditional(h, more ? 1u : 0u);
}

template <int D, int S> cudaError_t launch_loop_t(gbmd_engine* e, cudaStream_t s) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(e->loop_blocks);
    cfg.blockDim = dim3(128);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative; // every block resident at once: the grid barrier needs it
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_force_loop<D, S>, e->P, (Rec<D>*)e->pos[e->cur], (Rec<D>*)e->pos[e->cur ^ 1], e->qpos[e->cur],
                              e->qpos[e->cur ^ 1], e->vel, (const uint32_t*)e->nbr, (const uint32_t*)e->nbr_count,
                              (const Rec<D>*)e->ref_pos, e->ctl, e->block_steps);
}
template <int D> const void* loop_kernel(uint32_t S) {
    switch (S) {
    case 16: return (const void*)k_force_loop<D, 16>;
    case 8: return (const void*)k_force_loop<D, 8>;
    case 4: return (const void*)k_force_loop<D, 4>;
    case 2: return (const void*)k_force_loop<D, 2>;
    default: return (const void*)k_force_loop<D, 1>;
    }
}
template <int D> cudaError_t enqueue_loop_d(gbmd_engine* e, cudaStream_t s) {
    switch (e->loop_lanes) {
    case 16: return launch_loop_t<D, 16>(e, s);
    case 8: return launch_loop_t<D, 8>(e, s);
    case 4: return launch_loop_t<D, 4>(e, s);
    case 2: return launch_loop_t<D, 2>(e, s);
    default: return launch_loop_t<D, 1>(e, s);
    }
}
cudaError_t enqueue_loop(gbmd_engine* e, cudaStream_t s) {
    note_launch();
    return e->D == 2 ? enqueue_loop_d<2>(e, s) : enqueue_loop_d<3>(e, s);
}

// The persistent loop replaces per-step graph nodes for systems whose force grid fits on the GPU
// at once (one species, sigma = 1, f32 chain, no thermostat): the per-step conditional rebuild
// node alone costs more than the whole step of a small system. Lanes per particle as the step
// kernel's; fewer if the grid would not be resident.
int setup_step_loop(gbmd_engine* e) {
    e->loop_lanes = 0;
    if (!e->verlet || e->half || e->multi || e->opt.arith != GBMD_ARITH_F32 || e->P.int_mode || e->opt.rescale_every || e->P.bath || e->P.walls || e->P.bonds ||
        (e->opt.flags & GBMD_FLAG_NO_STEP_LOOP))
        return GBMD_OK;
    // Larger systems' steps are long enough that the graph's per-step nodes cost less than the
    // loop's barrier (3D N = 131,072: 71 us per step in graphs, 76 in the loop; 65,536: 53 vs 49).
    if (e->n >= STEP_LOOP_BELOW) return GBMD_OK;
    if (!(e->P.pc[0].sigma2s == 0x1p56f)) return GBMD_OK;
    int coop = 0, sms = 0;
    GBMD_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, e->opt.device));
    GBMD_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e->opt.device));
    if (!coop) return GBMD_OK;
    const uint32_t first = force_lanes(e);
    for (uint32_t S = first; S >= 1; S >>= 1) {
        int per = 0;
        GBMD_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, e->D == 2 ? loop_kernel<2>(S) : loop_kernel<3>(S), 128, 0));
        const uint64_t blocks = ((uint64_t)e->n * S + 127) / 128;
        // (one launch takes at most block_steps steps, and its grid barrier counts up to
        // steps x blocks arrivals in the low 32 bits of a 64-bit word, cleared per launch)
        if ((uint64_t)e->block_steps * blocks >= (1ull << 32)) continue;
        if (blocks >= 1 && blocks <= (uint64_t)per * (uint64_t)sms) {
            e->loop_lanes = S;
            e->loop_blocks = (uint32_t)blocks;
            return GBMD_OK;
        }
    }
    return GBMD_OK;
}

// kind 4: [k_loop_begin] -> WHILE (steps left) { [set IF] -> IF (trigger) { rebuild } -> the loop
// launch -> [set WHILE] }.
int capture_loop_block(gbmd_engine* e, cudaStream_t s, uint32_t target, uint64_t* body) {
    k_loop_begin<<<1, 1, 0, s>>>(e->ctl);
    note_launch();
    cudaStreamCaptureStatus status;
    cudaGraph_t g;
    const cudaGraphNode_t* deps;
    const cudaGraphEdgeData* edges;
    size_t ndeps;
    GBMD_CUDA_TRY(cudaStreamGetCaptureInfo(s, &status, nullptr, &g, &deps, &edges, &ndeps));
    cudaGraphConditionalHandle hw;
    GBMD_CUDA_TRY(cudaGraphConditionalHandleCreate(&hw, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams wp{};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = hw;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode;
    GBMD_CUDA_TRY(cudaGraphAddNode(&wnode, g, deps, edges, ndeps, &wp));
    GBMD_CUDA_TRY(cudaStreamBeginCaptureToGraph(e->st_body, wp.conditional.phGraph_out[0], nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    cudaGraph_t gb;
    GBMD_CUDA_TRY(cudaStreamGetCaptureInfo(e->st_body, &status, nullptr, &gb, &deps, &edges, &ndeps));
    cudaGraphConditionalHandle hi;
    GBMD_CUDA_TRY(cudaGraphConditionalHandleCreate(&hi, gb, 0, 0));
    k_set_cond<<<1, 1, 0, e->st_body>>>(hi, e->ctl);
    note_launch();
    GBMD_CUDA_TRY(cudaStreamGetCaptureInfo(e->st_body, &status, nullptr, &gb, &deps, &edges, &ndeps));
    cudaGraphNodeParams ip{};
    ip.type = cudaGraphNodeTypeConditional;
    ip.conditional.handle = hi;
    ip.conditional.type = cudaGraphCondTypeIf;
    ip.conditional.size = 1;
    cudaGraphNode_t inode;
    GBMD_CUDA_TRY(cudaGraphAddNode(&inode, gb, deps, edges, ndeps, &ip));
    GBMD_CUDA_TRY(cudaStreamBeginCaptureToGraph(e->st_body2, ip.conditional.phGraph_out[0], nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    const uint64_t b0 = launch_total();
    enqueue_rebuild(e, e->st_body2);
    *body = launch_total() - b0;
    cudaGraph_t tmp;
    GBMD_CUDA_TRY(cudaStreamEndCapture(e->st_body2, &tmp));
    GBMD_CUDA_TRY(cudaStreamUpdateCaptureDependencies(e->st_body, &inode, nullptr, 1, cudaStreamSetCaptureDependencies));
    GBMD_CUDA_TRY(enqueue_loop(e, e->st_body));
    k_set_while<<<1, 1, 0, e->st_body>>>(hw, e->ctl, target);
    note_launch();
    GBMD_CUDA_TRY(cudaStreamEndCapture(e->st_body, &tmp));
    GBMD_CUDA_TRY(cudaStreamUpdateCaptureDependencies(s, &wnode, nullptr, 1, cudaStreamSetCaptureDependencies));
    return GBMD_OK;
}

// Capture `count` steps starting at parity `parity` into a graph. kind 1 applies the thermostat
// after every rescale_every-th step of the block (blocks start on a thermostat boundary); kind 2
// applies it after its single step.
int capture_steps(gbmd_engine* e, int parity, uint32_t count, int kind, cudaGraphExec_t* out, uint64_t* launches) {
    int saved_cur = e->cur;
    e->cur = parity;
    uint64_t l0 = launch_total();
    cudaStream_t s = e->st;
    GBMD_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    uint64_t body = 0;
    if (kind == 4) {
        GBMD_TRY(capture_loop_block(e, s, count, &body));
        g_launches -= body; // counted per rebuild instead
    }
    for (uint32_t k = 0; k < (kind == 3 ? 1u : (kind == 4 ? 0u : count)); k++) {
        if (e->verlet) {
            cudaStreamCaptureStatus status;
            cudaGraph_t g;
            const cudaGraphNode_t* deps;
            const cudaGraphEdgeData* edges;
            size_t ndeps;
            GBMD_CUDA_TRY(cudaStreamGetCaptureInfo(s, &status, nullptr, &g, &deps, &edges, &ndeps));
            cudaGraphConditionalHandle h;
            GBMD_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
            k_set_cond<<<1, 1, 0, s>>>(h, e->ctl);
            note_launch();
            GBMD_CUDA_TRY(cudaStreamGetCaptureInfo(s, &status, nullptr, &g, &deps, &edges, &ndeps));
            cudaGraphNodeParams cp{};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = h;
            cp.conditional.type = cudaGraphCondTypeIf;
            cp.conditional.size = 1;
            cudaGraphNode_t node;
            GBMD_CUDA_TRY(cudaGraphAddNode(&node, g, deps, edges, ndeps, &cp));
            cudaGraph_t bodyg = cp.conditional.phGraph_out[0];
            GBMD_CUDA_TRY(cudaStreamBeginCaptureToGraph(e->st_body, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
            uint64_t b0 = launch_total();
            enqueue_rebuild(e, e->st_body);
            body = launch_total() - b0;
            g_launches -= body; // counted per replay instead
            cudaGraph_t tmp;
            GBMD_CUDA_TRY(cudaStreamEndCapture(e->st_body, &tmp));
            GBMD_CUDA_TRY(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
        }
        if (kind == 3) break; // the conditional rebuild alone
        enqueue_force(e, s);
        uint32_t every = e->opt.rescale_every;
        if ((kind == 1 && every && (k + 1) % every == 0) || kind == 2) enqueue_thermo(e, s);
    }
    cudaGraph_t graph;
    cudaError_t err = cudaStreamEndCapture(s, &graph);
    if (err != cudaSuccess) {
        e->cur = saved_cur;
        return fail(GBMD_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(err));
    }
    err = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (err != cudaSuccess) {
        e->cur = saved_cur;
        return fail(GBMD_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(err));
    }
    *launches = launch_total() - l0;
    g_launches -= *launches; // launches are counted when the graph is replayed
    if (kind == 4) *launches = 1; // k_loop_begin; three per WHILE iteration are counted from the device
    e->body_launches = body;
    e->cur = saved_cur;
    return GBMD_OK;
}

int run_graph(gbmd_engine* e, int which) {
    int parity = e->cur;
    uint32_t count = (which == 1 || which == 4) ? e->block_steps : (which == 3 ? 0u : 1u);
    if (!e->exec[parity][which]) {
        GBMD_TRY(capture_steps(e, parity, count, which, &e->exec[parity][which], &e->exec_launches[parity][which]));
    }
    GBMD_CUDA_TRY(cudaGraphLaunch(e->exec[parity][which], e->st));
    e->tcount += count;
    note_launch(e->exec_launches[parity][which]);
    e->launches += e->exec_launches[parity][which];
    if (e->verlet && (count & 1) && which != 4) e->cur ^= 1; // (the loop ends in its home buffer)
    return GBMD_OK;
}

// Bring the pair structure up to date for kicks and observables between steps: a Verlet list is
// rebuilt only if the displacement trigger has fired since the last build (the same device flag
// and conditional graph node the steps use), a cell list binned into the scratch state.
int prepare_pairs_cond(gbmd_engine* e) {
    if (e->half) {
        // the instruments walk full lists: build one now, and have the next step rebuild the
        // half-shell list it steps with (the trajectory does not depend on the storage order)
        enqueue_rebuild(e, e->st, true);
        k_set_trigger<<<1, 1, 0, e->st>>>(e->ctl);
        note_launch();
        GBMD_CUDA_TRY(cudaGetLastError());
        return GBMD_OK;
    }
    if (!e->verlet) {
        if (e->D == 2) enqueue_bin<2>(e, e->st, e->P);
        else enqueue_bin<3>(e, e->st, e->P);
        GBMD_CUDA_TRY(cudaGetLastError());
        return GBMD_OK;
    }
    return run_graph(e, 3);
}
// The same with the Verlet list always rebuilt (the positions wrapped into the box, the
// storage re-sorted).
int prepare_pairs(gbmd_engine* e) {
    if (e->verlet) {
        enqueue_rebuild(e, e->st);
    } else {
        if (e->D == 2) enqueue_bin<2>(e, e->st, e->P);
        else enqueue_bin<3>(e, e->st, e->P);
    }
    GBMD_CUDA_TRY(cudaGetLastError());
    return GBMD_OK;
}

// Kicks (storage order) and the per-block observables at the current positions; optionally
// reverse the velocities. Cell mode works on (and copies back) the sorted scratch state.
template <int D, bool MULTI, bool INT> void kicks_launch(gbmd_engine* e, int32_t* kicks, double* partial, int reverse) {
    uint32_t threads = 128;
    uint32_t nb = blocks_for(e->n, threads);
    if (e->P.bonds) {
        k_slot_of<<<blocks_for(e->n, 256), 256, 0, e->st>>>(e->n, e->verlet ? e->ids : e->ids_scr, e->slot_of);
        note_launch();
    }
    if (e->verlet)
        k_kicks<D, MULTI, INT><<<nb, threads, 0, e->st>>>(e->P, (const Rec<D>*)e->pos[e->cur], e->species, e->ids, e->nbr, e->nbr_count,
                                                          nullptr, nullptr, e->vel, kicks, partial, reverse);
    else
        k_kicks<D, MULTI, INT><<<nb, threads, 0, e->st>>>(e->P, (const Rec<D>*)e->pos_scr, e->species_scr, e->ids_scr, nullptr, nullptr,
                                                          e->keys[e->sorted], e->start, e->vel_scr, kicks, partial, reverse);
}
template <int D, bool MULTI> int kicks_t(gbmd_engine* e, int32_t* kicks, double* partial, int reverse) {
    if (e->P.int_mode) kicks_launch<D, MULTI, true>(e, kicks, partial, reverse);
    else kicks_launch<D, MULTI, false>(e, kicks, partial, reverse);
    if (reverse && e->P.piston_drive) {
        k_piston_reverse<<<1, 1, 0, e->st>>>(e->P);
        note_launch();
    }
    if (!e->verlet) {
        // positions, velocities and ids live in scratch (sorted) until copied back
        GBMD_CUDA_TRY(cudaMemcpyAsync(e->pos[e->cur], e->pos_scr, (size_t)e->n * e->rec, cudaMemcpyDeviceToDevice, e->st));
        GBMD_CUDA_TRY(cudaMemcpyAsync(e->vel, e->vel_scr, (size_t)e->n * D * 4, cudaMemcpyDeviceToDevice, e->st));
        GBMD_CUDA_TRY(cudaMemcpyAsync(e->species, e->species_scr, (size_t)e->n * 4, cudaMemcpyDeviceToDevice, e->st));
        GBMD_CUDA_TRY(cudaMemcpyAsync(e->ids, e->ids_scr, (size_t)e->n * 4, cudaMemcpyDeviceToDevice, e->st));
    }
    note_launch();
    GBMD_CUDA_TRY(cudaGetLastError());
    return GBMD_OK;
}
int kicks_dispatch(gbmd_engine* e, int32_t* kicks, double* partial, int reverse) {
    if (e->D == 2) return e->multi ? kicks_t<2, true>(e, kicks, partial, reverse) : kicks_t<2, false>(e, kicks, partial, reverse);
    return e->multi ? kicks_t<3, true>(e, kicks, partial, reverse) : kicks_t<3, false>(e, kicks, partial, reverse);
}

// ---- id-ordered I/O
struct Box3 {
    int64_t v[3];
    __device__ int64_t operator[](int a) const { return v[a]; }
};
template <int D>
__global__ void k_to_ids(uint32_t n, Box3 box, const Rec<D>* pos, const int32_t* vel, const uint32_t* species, const uint32_t* ids,
                         int64_t* opos, int32_t* ovel, uint32_t* ospecies) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    uint32_t id = ids[s];
    int64_t x[3];
    load_particle<D, false>(pos, nullptr, s, x);
    for (int a = 0; a < D; a++) {
        opos[(size_t)D * id + a] = wrap(x[a], box[a]);
        ovel[(size_t)D * id + a] = vel[D * s + a];
    }
    ospecies[id] = species[s];
}
template <int D>
__global__ void k_from_ids(uint32_t n, const int64_t* ipos, const int32_t* ivel, const uint32_t* ispecies, Rec<D>* pos, int32_t* vel,
                           uint32_t* species, uint32_t* ids) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int64_t x[3];
    for (int a = 0; a < D; a++) {
        x[a] = ipos[(size_t)D * s + a];
        vel[D * s + a] = ivel[(size_t)D * s + a];
    }
    store_pos<D>(pos, s, x, ispecies[s]);
    species[s] = ispecies[s];
    ids[s] = s;
}
__global__ void k_scatter_i32(uint32_t n, uint32_t d, const uint32_t* ids, const int32_t* in, int32_t* out) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    for (uint32_t a = 0; a < d; a++) out[(size_t)d * ids[s] + a] = in[(size_t)d * s + a];
}
template <int D> __global__ void k_flip(uint32_t n, const uint32_t* ids, uint32_t id, uint32_t axis, uint32_t bit, Rec<D>* pos) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n || ids[s] != id) return;
    long long* p = reinterpret_cast<long long*>(pos + s);
    p[axis] ^= (long long)(1ull << bit);
}
// GpuEngine::flip_species_bit (engine.rs:1014-1024): the same bit of every particle whose species
// is in the mask.
template <int D>
__global__ void k_flip_species(uint32_t n, const uint32_t* species, uint32_t mask, uint32_t axis, uint32_t bit, Rec<D>* pos) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n || !((mask >> species[s]) & 1u)) return;
    long long* p = reinterpret_cast<long long*>(pos + s);
    p[axis] ^= (long long)(1ull << bit);
}

// ---- page commands (md::GpuEngine, crates/md/src/engine.rs:1026-1063)
struct RegionCmd {
    float lo[3], hi[3];
    float scale;
    int32_t add[3];
};
// md.wgsl:216-229 / md3.wgsl:541-553: for every unpinned particle whose coord_f32 position
// (f32(x >> 32) + f32(x & 0xffffffff) 2^-32, of the wrapped position) is inside [lo, hi):
// v <- rint(f32(v) scale) + add per axis, the sum wrapping.
template <int D> __global__ void k_kick_region(Params P, const Rec<D>* pos, const uint32_t* species, int32_t* vel, RegionCmd C) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P.n || ((P.pinned >> species[s]) & 1u)) return;
    int64_t x[3];
    load_particle<D, false>(pos, nullptr, s, x);
#pragma unroll
    for (int a = 0; a < D; a++) {
        const uint64_t w = (uint64_t)wrap(x[a], P.box[a]);
        const float c = __fadd_rn(__uint2float_rn((uint32_t)(w >> 32)), __fmul_rn(__uint2float_rn((uint32_t)w), 0x1p-32f));
        if (c < C.lo[a] || c >= C.hi[a]) return;
    }
#pragma unroll
    for (int a = 0; a < D; a++) vel[D * s + a] = wadd(__float2int_rn(__fmul_rn(__int2float_rn(vel[D * s + a]), C.scale)), C.add[a]);
}
// reorder.wgsl:80-99 / md3.wgsl:556-574: the particles whose ids are in the sorted `list` take
// species `to` (in the species array, the 3D record's fourth word and the quotient record's top byte).
template <int D>
__global__ void k_set_species(uint32_t n, const uint32_t* ids, const uint32_t* list, uint32_t count, uint32_t to, uint32_t* species, Rec<D>* pos,
                              uint4* qpos) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t id = ids[s];
    uint32_t lo = 0, hi = count;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) / 2;
        if (list[mid] < id) lo = mid + 1;
        else hi = mid;
    }
    if (lo >= count || list[lo] != id) return;
    species[s] = to;
    if constexpr (D == 3) reinterpret_cast<long long*>(pos + s)[3] = (long long)to;
    if (qpos) qpos[s].w = (qpos[s].w & 0x00ffffffu) | (to << 24);
}
// md.wgsl:151-156 / md3.wgsl:655-660: every particle of species `sp` gets velocity v.
__global__ void k_set_species_velocity(uint32_t n, uint32_t dim, const uint32_t* species, uint32_t sp, int3 v, int32_t* vel) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n || species[s] != sp) return;
    vel[dim * s] = v.x;
    vel[dim * s + 1] = v.y;
    if (dim == 3) vel[dim * s + 2] = v.z;
}
int upload_state(gbmd_engine* e, const int64_t* pos, const int32_t* vel, const uint32_t* species) {
    size_t n = e->n, D = e->D;
    for (size_t i = 0; i < n; i++)
        if (species[i] >= e->sys.nspecies) return fail(GBMD_E_INVALID, "species index out of range");
    for (size_t i = 0; i < n; i++)
        for (size_t a = 0; a < D; a++)
            if (pos[D * i + a] < 0 || pos[D * i + a] >= e->sys.box_len[a])
                return fail(GBMD_E_INVALID, "positions must lie in [0, L) on every axis");
    GBMD_CUDA_TRY(cudaMemcpyAsync(e->staging, pos, n * D * 8, cudaMemcpyHostToDevice, e->st));
    GBMD_CUDA_TRY(cudaMemcpyAsync(e->staging_v, vel, n * D * 4, cudaMemcpyHostToDevice, e->st));
    GBMD_CUDA_TRY(cudaMemcpyAsync(e->staging_s, species, n * 4, cudaMemcpyHostToDevice, e->st));
    if (D == 2)
        k_from_ids<2><<<blocks_for(n, 256), 256, 0, e->st>>>((uint32_t)n, (const int64_t*)e->staging, e->staging_v, e->staging_s,
                                                            (Rec<2>*)e->pos[e->cur], e->vel, e->species, e->ids);
    else
        k_from_ids<3><<<blocks_for(n, 256), 256, 0, e->st>>>((uint32_t)n, (const int64_t*)e->staging, e->staging_v, e->staging_s,
                                                            (Rec<3>*)e->pos[e->cur], e->vel, e->species, e->ids);
    note_launch();
    uint32_t one = 1;
    GBMD_CUDA_TRY(cudaMemcpyAsync(e->ctl, &one, 4, cudaMemcpyHostToDevice, e->st));
    GBMD_CUDA_TRY(cudaStreamSynchronize(e->st));
    return upload_ranks(e, species);
}

int read_state_dev(gbmd_engine* e) {
    size_t n = e->n;
    Box3 box{{e->P.box[0], e->P.box[1], e->P.box[2]}};
    if (e->D == 2)
        k_to_ids<2><<<blocks_for(n, 256), 256, 0, e->st>>>((uint32_t)n, box, (const Rec<2>*)e->pos[e->cur], e->vel, e->species, e->ids,
                                                          (int64_t*)e->staging, e->staging_v, e->staging_s);
    else
        k_to_ids<3><<<blocks_for(n, 256), 256, 0, e->st>>>((uint32_t)n, box, (const Rec<3>*)e->pos[e->cur], e->vel, e->species, e->ids,
                                                          (int64_t*)e->staging, e->staging_v, e->staging_s);
    note_launch();
    GBMD_CUDA_TRY(cudaGetLastError());
    return GBMD_OK;
}

int check_ctl(gbmd_engine* e) {
    uint32_t c[11];
    GBMD_CUDA_TRY(cudaMemcpyAsync(c, e->ctl, sizeof(c), cudaMemcpyDeviceToHost, e->st));
    GBMD_CUDA_TRY(cudaStreamSynchronize(e->st));
    e->last_rebuilds = c[2];
    e->loop_iters = c[CTL_LOOP_ITERS];
    if (c[CTL_LOOP_ERR]) {
        e->failed = true;
        return fail(GBMD_E_TIMEOUT, "a grid barrier of the persistent step loop ran out of time");
    }
    if (c[1]) {
        e->failed = true;
        return fail(GBMD_E_OVERFLOW, "a Verlet list overflowed its capacity (raise gbmd_options.cap)");
    }
    return GBMD_OK;
}

int create_common(gbmd_engine* e, const gbmd_system* sys, uint32_t n, const gbmd_options* opts) {
    e->live = true;
    g_live_engines++;
    e->sys = *sys;
    if (opts) e->opt = *opts;
    e->n = n;
    e->D = (int)sys->dim;
    e->multi = sys->nspecies > 1;
    e->rec = e->D == 2 ? 16 : 32;
    int mode = e->opt.mode;
    if (mode == GBMD_MODE_AUTO) mode = (e->D == 2 && n < 24000) ? GBMD_MODE_CELLS : GBMD_MODE_VERLET; // ForceMode::auto
    e->verlet = mode == GBMD_MODE_VERLET;
    if (e->opt.arith != GBMD_ARITH_F32 && e->opt.arith != GBMD_ARITH_INT) return fail(GBMD_E_INVALID, "unknown pair arithmetic");
    e->skin = e->verlet ? (e->opt.skin > 0 ? e->opt.skin : 0.4) : 0.0;
    uint32_t nc[3];
    GBMD_TRY(cells_for(*sys, rc_max(*sys) + e->skin, nc));
    uint32_t cap = 0;
    if (e->verlet && n >= (1u << 26)) return fail(GBMD_E_UNSUPPORTED, "Verlet lists hold at most 2^26 particles per engine");
    if (e->verlet) {
        // ForceMode::verlet_with_skin's sizing (engine.rs:130-141), without the 128 MiB clamp
        double r = rc_max(*sys) + e->skin, vol = 1.0;
        for (int a = 0; a < e->D; a++) vol *= to_f64h(sys->box_len[a]);
        double density = (double)n / vol;
        double sphere = e->D == 2 ? M_PI * r * r : 4.0 / 3.0 * M_PI * r * r * r;
        cap = e->opt.cap ? e->opt.cap : (uint32_t)std::ceil(sphere * std::max(2.0 * density, 1.2)) + 8;
    }
    fill_params(e->P, *sys, n, e->skin, cap, nc);
    if (e->opt.flags & GBMD_FLAG_NO_PATH_BOUND) e->P.ub_thr = 0;
    if (e->verlet && e->D == 3 && !e->multi && e->opt.arith == GBMD_ARITH_F32 && !e->P.walls && (e->opt.flags & GBMD_FLAG_HALF_LISTS)) {
        // Half-shell lists address a neighbour by its offset in its row of cells (16 bits): rows
        // must stay far below 65,536 particles (the build reports an overflow otherwise). The
        // force step's shared-memory windows hold six mean rows with a tenth to spare; rows
        // beyond that accumulate in global memory.
        const double mean_row = (double)n / ((double)nc[1] * nc[2]);
        if (mean_row * 4.0 < 65536.0) {
            e->half = true;
            const uint32_t max_slots = (uint32_t)((55u * 1024u) / 12u); // four blocks per SM
            e->P.half_lists = 1;
            e->P.win_cap = std::min<uint32_t>(max_slots, (uint32_t)std::ceil(mean_row * HALF_WINDOWS * 1.1) + 64u);
        }
    }
    if (e->verlet && !e->half && !(e->opt.flags & GBMD_FLAG_WHOLE_CELLS) && list_build_lanes(e) > 1)
        set_sub_buckets(e->P, sys->dim, (rc_max(*sys) + e->skin) * (1.0 + 1e-4));
    e->block_steps = e->opt.block_steps ? e->opt.block_steps : 64;
    if (e->opt.rescale_every) {
        if (!(e->opt.rescale_t > 0.0)) return fail(GBMD_E_INVALID, "the rescale thermostat needs a positive temperature");
        uint32_t every = e->opt.rescale_every;
        e->block_steps = every * std::max<uint32_t>(1, e->block_steps / every);
    }
    e->thermo_nb = std::min<uint32_t>(std::max<uint32_t>(blocks_for(n, 256), 1), 512);
    GBMD_CUDA_TRY(cudaSetDevice(e->opt.device));
    keep_pool_memory(e->opt.device);
    GBMD_CUDA_TRY(cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking));
    GBMD_CUDA_TRY(cudaStreamCreateWithFlags(&e->st_body, cudaStreamNonBlocking));
    GBMD_CUDA_TRY(cudaStreamCreateWithFlags(&e->st_body2, cudaStreamNonBlocking));
    size_t D = e->D;
    GBMD_TRY(alloc(e, &e->pos[0], n * e->rec));
    GBMD_TRY(alloc(e, &e->pos[1], n * e->rec));
    GBMD_TRY(alloc(e, &e->pos_scr, n * e->rec));
    GBMD_TRY(alloc(e, &e->ref_pos, n * e->rec));
    GBMD_TRY(allocT(e, &e->vel, n * D));
    GBMD_TRY(allocT(e, &e->vel_scr, n * D));
    GBMD_TRY(allocT(e, &e->kicks, n * D));
    GBMD_TRY(allocT(e, &e->species, n));
    GBMD_TRY(allocT(e, &e->species_scr, n));
    GBMD_TRY(allocT(e, &e->ids, n));
    GBMD_TRY(allocT(e, &e->ids_scr, n));
    for (int b = 0; b < 2; b++) {
        GBMD_TRY(allocT(e, &e->keys[b], n));
        GBMD_TRY(allocT(e, &e->vals[b], n));
    }
    size_t hist_n = radix_hist_elems(n);
    GBMD_TRY(allocT(e, &e->hist, hist_n));
    GBMD_TRY(allocT(e, &e->scan_tmp, std::max(scan_tmp_elems(hist_n), scan_tmp_elems(n))));
    GBMD_TRY(allocT(e, &e->start, ((size_t)e->P.ncell << e->P.key_shift) + 1));
    if (e->verlet) {
        GBMD_TRY(allocT(e, &e->nbr, ((size_t)n + 31) / 32 * 32 * (((size_t)cap + 3) & ~(size_t)3)));
        GBMD_TRY(allocT(e, &e->nbr_count, n));
    }
    if (e->half) {
        GBMD_TRY(allocT(e, &e->acc, 4 * (size_t)n));
        GBMD_CUDA_TRY(cudaMemsetAsync(e->acc, 0, 16 * (size_t)n, e->st));
        const int smem = (int)(e->P.win_cap * 12);
        GBMD_CUDA_TRY(cudaFuncSetAttribute(k_force_half<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        GBMD_CUDA_TRY(cudaFuncSetAttribute(k_force_half<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    }
    GBMD_TRY(allocT(e, &e->ctl, 16));
    {
        // per ledger slot, one entry per compartment along its wall (the most on either axis)
        uint32_t pw = 1;
        for (uint32_t a = 0; a < 2 && e->D == 2; a++)
            if (e->P.comp_shift[a]) pw = std::max<uint32_t>(pw, (uint32_t)(e->sys.box_len[a] >> e->P.comp_shift[a]));
        e->P.ledger_per_wall = pw;
    }
    GBMD_TRY(allocT(e, &e->ledger, 3 * (size_t)GBMD_LEDGER_SLOTS * e->P.ledger_per_wall));
    e->P.ids_list = e->ids; // (the force kernel's scenario epilogue)
    e->P.ledger = e->ledger;
    e->P.clock_word = e->ctl + CTL_CLOCK;
    GBMD_CUDA_TRY(cudaMemsetAsync(e->ledger, 0, 24 * (size_t)GBMD_LEDGER_SLOTS * e->P.ledger_per_wall, e->st));
    if (e->opt.arith == GBMD_ARITH_INT) {
        std::vector<int32_t> tab;
        std::vector<double> pair4;
        uint32_t len = 0;
        int_tables(*sys, tab, len, e->P.irc2, pair4);
        GBMD_TRY(allocT(e, &e->itab, tab.size()));
        GBMD_TRY(allocT(e, &e->ipair, pair4.size()));
        GBMD_CUDA_TRY(cudaMemcpy(e->itab, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice));
        GBMD_CUDA_TRY(cudaMemcpy(e->ipair, pair4.data(), pair4.size() * 8, cudaMemcpyHostToDevice));
        e->P.int_mode = 1;
        e->P.itab_len = len;
        e->P.itab = e->itab;
        e->P.ipair = e->ipair;
    }
    GBMD_TRY(setup_step_loop(e)); // (after the pair arithmetic is settled: f32 engines only)
    GBMD_TRY(allocT(e, &e->relf, n));
    GBMD_TRY(allocT(e, &e->qpos[0], n));
    GBMD_TRY(allocT(e, &e->qpos[1], n));
    GBMD_TRY(allocT(e, &e->mrank, n));
    GBMD_TRY(allocT(e, &e->tpart, 8 * (size_t)e->thermo_nb));
    GBMD_TRY(allocT(e, &e->vpart, 3 * ((size_t)e->thermo_nb + 1))); // the block partials, then their total
    GBMD_TRY(allocT(e, &e->tfac, 2));
    GBMD_TRY(allocT(e, &e->partial, 4 * (size_t)blocks_for(n, 128) + 4));
    GBMD_TRY(alloc(e, &e->staging, n * D * 8));
    GBMD_TRY(allocT(e, &e->staging_v, n * D));
    GBMD_TRY(allocT(e, &e->staging_s, n));
    GBMD_CUDA_TRY(cudaMemsetAsync(e->ctl, 0, 64, e->st));
    return GBMD_OK;
}

} // namespace

// The pinned pool for the batches' frames.
namespace gbmd {
void* pinned_alloc(size_t bytes, size_t* cap) {
    *cap = pin_class(bytes);
    void* p = pinned_take(*cap);
    if (!p) *cap = 0;
    return p;
}
void pinned_release(void* p, size_t cap) { pinned_give(p, cap); }
} // namespace gbmd

// ================================================================== C ABI
extern "C" {

int gbmd_create(const gbmd_system* sys, const int64_t* pos, const int32_t* vel, const uint32_t* species, uint32_t n,
                const gbmd_options* opts, gbmd_engine** out) {
    if (!sys || !out || (n && (!pos || !vel || !species))) return fail(GBMD_E_INVALID, "null argument");
    *out = nullptr;
    GBMD_TRY(validate_system(*sys, n));
    if (n == 0) return fail(GBMD_E_INVALID, "an engine needs at least one particle");
    auto* e = new gbmd_engine;
    int r = create_common(e, sys, n, opts);
    if (r == GBMD_OK) r = upload_state(e, pos, vel, species);
    if (r != GBMD_OK) {
        std::string msg = t_error;
        free_all(e);
        delete e;
        return fail(r, msg);
    }
    *out = e;
    return GBMD_OK;
}

int gbmd_create_seeded(const gbmd_system* sys, const gbmd_init* spec, const gbmd_options* opts, gbmd_engine** out) {
    if (!sys || !spec || !out) return fail(GBMD_E_INVALID, "null argument");
    *out = nullptr;
    GBMD_TRY(validate_system(*sys, spec->n));
    if (spec->n == 0) return fail(GBMD_E_INVALID, "an engine needs at least one particle");
    auto* e = new gbmd_engine;
    int r = create_common(e, sys, spec->n, opts);
    if (r == GBMD_OK) r = init_state_device(*sys, *spec, e->pos[e->cur], e->vel, e->species, e->st);
    if (r == GBMD_OK) {
        iota(e->ids, e->n, e->st);
        note_launch();
        uint32_t one = 1;
        cudaMemcpyAsync(e->ctl, &one, 4, cudaMemcpyHostToDevice, e->st);
        if (cudaStreamSynchronize(e->st) != cudaSuccess) r = fail(GBMD_E_CUDA, "seeded init failed");
        if (r == GBMD_OK) {
            std::vector<uint32_t> zeros(e->n, 0); // the recipes create species 0 only
            r = upload_ranks(e, zeros.data());
        }
    }
    if (r != GBMD_OK) {
        std::string msg = t_error;
        free_all(e);
        delete e;
        return fail(r, msg);
    }
    *out = e;
    return GBMD_OK;
}

int gbmd_destroy(gbmd_engine* e) {
    if (!e) return GBMD_OK;
    cudaStreamSynchronize(e->st);
    free_all(e);
    delete e;
    return GBMD_OK;
}

int gbmd_step(gbmd_engine* e, uint64_t steps) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    if (e->failed) return fail(GBMD_E_OVERFLOW, "the engine is in a failed state (a list overflowed, or a step-loop barrier ran out); gbmd_upload a state to continue");
    uint64_t left = steps;
    uint32_t every = e->opt.rescale_every;
    if (e->P.bath && steps) { // the device clock follows the host's (uploads, snapshots, reversals)
        k_clock_set<<<1, 1, 0, e->st>>>(e->ctl, e->clock);
        note_launch();
    }
    while (left > 0) {
        bool aligned = every == 0 || e->tcount % every == 0;
        if (aligned && left >= e->block_steps) {
            GBMD_TRY(run_graph(e, e->loop_lanes && g_live_engines.load() == 1 ? 4 : 1));
            left -= e->block_steps;
        } else {
            bool thermo = every && (e->tcount + 1) % every == 0;
            GBMD_TRY(run_graph(e, thermo ? 2 : 0));
            left--;
        }
    }
    e->steps += (int64_t)steps;
    e->clock += (uint32_t)steps;
    GBMD_CUDA_TRY(cudaGetLastError());
    return GBMD_OK;
}

int gbmd_sync(gbmd_engine* e) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    GBMD_CUDA_TRY(cudaStreamSynchronize(e->st));
    return check_ctl(e);
}

int gbmd_reverse(gbmd_engine* e) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    GBMD_TRY(prepare_pairs_cond(e));
    GBMD_TRY(kicks_dispatch(e, nullptr, nullptr, 1));
    e->steps = -e->steps;
    return gbmd_sync(e);
}

int gbmd_read_state(gbmd_engine* e, int64_t* pos, int32_t* vel, uint32_t* species) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    GBMD_TRY(read_state_dev(e));
    size_t n = e->n, D = e->D;
    if (pos) GBMD_CUDA_TRY(cudaMemcpyAsync(pos, e->staging, n * D * 8, cudaMemcpyDeviceToHost, e->st));
    if (vel) GBMD_CUDA_TRY(cudaMemcpyAsync(vel, e->staging_v, n * D * 4, cudaMemcpyDeviceToHost, e->st));
    if (species) GBMD_CUDA_TRY(cudaMemcpyAsync(species, e->staging_s, n * 4, cudaMemcpyDeviceToHost, e->st));
    return gbmd_sync(e);
}

int gbmd_read_kinetic(gbmd_engine* e, double* kinetic, uint32_t* species, double* total) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    GBMD_TRY(read_state_dev(e));
    const size_t n = e->n, D = e->D;
    std::vector<int32_t> vel(n * D);
    std::vector<uint32_t> sp(n);
    GBMD_CUDA_TRY(cudaMemcpyAsync(vel.data(), e->staging_v, n * D * 4, cudaMemcpyDeviceToHost, e->st));
    GBMD_CUDA_TRY(cudaMemcpyAsync(sp.data(), e->staging_s, n * 4, cudaMemcpyDeviceToHost, e->st));
    GBMD_TRY(gbmd_sync(e));
    double sum = 0.0;
    for (size_t i = 0; i < n; i++) { // 1/2 m |v|^2, v = velocity(v) = v UNIT / dt (system.rs:423-425)
        double k = 0.0;
        for (size_t a = 0; a < D; a++) {
            const double u = (double)vel[D * i + a] * (1.0 / 4294967296.0) / e->sys.dt;
            k += u * u;
        }
        k *= ((e->sys.pinned >> sp[i]) & 1u) ? 0.0 : 0.5 * e->sys.masses[sp[i]]; // pinned: 0 (observe.wgsl:55)
        if (kinetic) kinetic[i] = k;
        if (species) species[i] = sp[i];
        sum += k;
    }
    if (total) *total = sum;
    return GBMD_OK;
}

int gbmd_upload(gbmd_engine* e, const int64_t* pos, const int32_t* vel, const uint32_t* species) {
    if (!e || !pos || !vel || !species) return fail(GBMD_E_INVALID, "null argument");
    GBMD_CUDA_TRY(cudaStreamSynchronize(e->st));
    e->failed = false;
    uint32_t zero[2] = {0, 0};
    GBMD_CUDA_TRY(cudaMemcpyAsync(e->ctl, zero, 8, cudaMemcpyHostToDevice, e->st));
    // the step loop's words (steps done, barrier, error, WHILE count), as at creation
    GBMD_CUDA_TRY(cudaMemsetAsync(e->ctl + CTL_LOOP_DONE, 0, (CTL_BAR_ARRIVE + 2 - CTL_LOOP_DONE) * 4, e->st));
    return upload_state(e, pos, vel, species);
}

int gbmd_kicks(gbmd_engine* e, int32_t* kicks, double* potential) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    GBMD_TRY(prepare_pairs_cond(e));
    GBMD_TRY(kicks_dispatch(e, e->kicks, e->partial, 0));
    size_t n = e->n;
    if (kicks) {
        k_scatter_i32<<<blocks_for(n, 256), 256, 0, e->st>>>((uint32_t)n, e->D, e->ids, e->kicks, (int32_t*)e->staging_v);
        note_launch();
        GBMD_CUDA_TRY(cudaMemcpyAsync(kicks, e->staging_v, n * e->D * 4, cudaMemcpyDeviceToHost, e->st));
    }
    uint32_t nb = blocks_for(n, 128);
    std::vector<double> part(4 * (size_t)nb);
    GBMD_CUDA_TRY(cudaMemcpyAsync(part.data(), e->partial, part.size() * 8, cudaMemcpyDeviceToHost, e->st));
    GBMD_TRY(gbmd_sync(e));
    if (potential) {
        double pe = 0.0;
        for (uint32_t b = 0; b < nb; b++) pe += part[4 * b];
        *potential = pe;
    }
    return GBMD_OK;
}

// The same kicks with f64 pair arithmetic (IntEngine<f64>): the accuracy reference of the f32
// path, on the device so that it runs at full size.
int gbmd_kicks_f64(gbmd_engine* e, int32_t* kicks, double* potential) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    if (e->P.walls || e->P.bonds) return fail(GBMD_E_UNSUPPORTED, "the f64 reference kicks are for periodic pair systems");
    GBMD_TRY(prepare_pairs_cond(e));
    PairsF64 Q;
    std::memset(&Q, 0, sizeof(Q));
    const gbmd_system& s = e->sys;
    for (uint32_t a = 0; a < s.nspecies; a++) {
        Q.kick_c[a] = ((s.pinned >> a) & 1u) ? 0.0 : s.dt * s.dt / s.masses[a] * 4294967296.0;
        for (uint32_t b = 0; b < s.nspecies; b++) {
            const gbmd_pair& p = s.pairs[a * s.nspecies + b];
            uint32_t q = a * e->P.ns + b;
            Q.rc2[q] = p.rc * p.rc;
            Q.eps4[q] = 4.0 * p.eps;
            Q.sigma2[q] = p.sigma * p.sigma;
            Q.shift[q] = pair_shift(p);
            Q.six_eps4[q] = 6.0 * Q.eps4[q];
        }
    }
    size_t n = e->n;
    double* pe_dev = nullptr;
    if (cudaMallocAsync((void**)&pe_dev, n * 8, e->st) != cudaSuccess) return fail(GBMD_E_NOMEM, "f64 potential");
    uint32_t nb = blocks_for(e->n, 128);
    const bool cells = !e->verlet;
    const void* pos = cells ? e->pos_scr : e->pos[e->cur];
    const uint32_t* sp = cells ? e->species_scr : e->species;
    const uint32_t* ids = cells ? e->ids_scr : e->ids;
    const uint32_t* nbr = cells ? nullptr : e->nbr;
    const uint32_t* cnt = cells ? nullptr : e->nbr_count;
    const uint32_t* keys = cells ? e->keys[e->sorted] : nullptr;
    const uint32_t* st = cells ? e->start : nullptr;
#define GBMD_KF64(DD, MM) \
    k_kicks_f64<DD, MM><<<nb, 128, 0, e->st>>>(e->P, Q, (const Rec<DD>*)pos, sp, nbr, cnt, keys, st, e->kicks, pe_dev)
    if (e->D == 2) {
        if (e->multi) GBMD_KF64(2, true);
        else GBMD_KF64(2, false);
    } else {
        if (e->multi) GBMD_KF64(3, true);
        else GBMD_KF64(3, false);
    }
#undef GBMD_KF64
    note_launch();
    int rc = GBMD_OK;
    std::vector<double> pe_host(potential ? n : 0);
    if (kicks) {
        k_scatter_i32<<<blocks_for(n, 256), 256, 0, e->st>>>((uint32_t)n, e->D, ids, e->kicks, (int32_t*)e->staging_v);
        note_launch();
        if (cudaMemcpyAsync(kicks, e->staging_v, n * e->D * 4, cudaMemcpyDeviceToHost, e->st) != cudaSuccess) rc = fail(GBMD_E_CUDA, "kicks copy");
    }
    if (rc == GBMD_OK && potential && cudaMemcpyAsync(pe_host.data(), pe_dev, n * 8, cudaMemcpyDeviceToHost, e->st) != cudaSuccess)
        rc = fail(GBMD_E_CUDA, "potential copy");
    cudaFreeAsync(pe_dev, e->st);
    cudaError_t err = cudaStreamSynchronize(e->st);
    if (rc != GBMD_OK) return rc;
    if (err != cudaSuccess) return fail(GBMD_E_CUDA, cudaGetErrorString(err));
    if (potential) {
        double pe = 0.0;
        for (size_t i = 0; i < n; i++) pe += pe_host[i];
        *potential = pe;
    }
    return GBMD_OK;
}

int gbmd_flip_bit(gbmd_engine* e, uint32_t id, uint32_t axis, uint32_t bit) {
    if (!e || id >= e->n || axis >= (uint32_t)e->D || bit > 62) return fail(GBMD_E_INVALID, "bad flip_bit argument");
    GBMD_TRY(prepare_pairs(e)); // wraps the positions into the box (they drift out between list builds)
    if (e->D == 2) k_flip<2><<<blocks_for(e->n, 256), 256, 0, e->st>>>(e->n, e->ids, id, axis, bit, (Rec<2>*)e->pos[e->cur]);
    else k_flip<3><<<blocks_for(e->n, 256), 256, 0, e->st>>>(e->n, e->ids, id, axis, bit, (Rec<3>*)e->pos[e->cur]);
    note_launch();
    uint32_t one = 1;
    GBMD_CUDA_TRY(cudaMemcpyAsync(e->ctl, &one, 4, cudaMemcpyHostToDevice, e->st));
    return gbmd_sync(e);
}

int gbmd_kick_region(gbmd_engine* e, const double* lo, const double* hi, double scale, const double* add) {
    if (!e || !lo || !hi || !add) return fail(GBMD_E_INVALID, "null argument");
    RegionCmd C{};
    for (int a = 0; a < 3; a++) {
        C.lo[a] = a < e->D ? (float)lo[a] : 0.0f;
        C.hi[a] = a < e->D ? (float)hi[a] : 0.0f;
        C.add[a] = a < e->D ? to_step_displacement(e->sys, add[a]) : 0;
    }
    C.scale = (float)scale;
    if (e->D == 2) k_kick_region<2><<<blocks_for(e->n, 256), 256, 0, e->st>>>(e->P, (const Rec<2>*)e->pos[e->cur], e->species, e->vel, C);
    else k_kick_region<3><<<blocks_for(e->n, 256), 256, 0, e->st>>>(e->P, (const Rec<3>*)e->pos[e->cur], e->species, e->vel, C);
    note_launch();
    GBMD_CUDA_TRY(cudaGetLastError());
    return GBMD_OK;
}

int gbmd_set_species(gbmd_engine* e, const uint32_t* ids, uint32_t count, uint32_t species) {
    if (!e || (count && !ids)) return fail(GBMD_E_INVALID, "null argument");
    if (species >= e->sys.nspecies) return fail(GBMD_E_INVALID, "species index out of range");
    if (count == 0) return GBMD_OK;
    std::vector<uint32_t> list(ids, ids + count);
    std::sort(list.begin(), list.end());
    list.erase(std::unique(list.begin(), list.end()), list.end());
    if (list.back() >= e->n) return fail(GBMD_E_INVALID, "particle id out of range");
    uint32_t* d_list = nullptr;
    if (cudaMallocAsync((void**)&d_list, list.size() * 4, e->st) != cudaSuccess) return fail(GBMD_E_NOMEM, "set_species list");
    GBMD_CUDA_TRY(cudaMemcpyAsync(d_list, list.data(), list.size() * 4, cudaMemcpyHostToDevice, e->st));
    const uint32_t m = (uint32_t)list.size();
    if (e->D == 2)
        k_set_species<2><<<blocks_for(e->n, 256), 256, 0, e->st>>>(e->n, e->ids, d_list, m, species, e->species, (Rec<2>*)e->pos[e->cur],
                                                                    e->verlet ? e->qpos[e->cur] : nullptr);
    else
        k_set_species<3><<<blocks_for(e->n, 256), 256, 0, e->st>>>(e->n, e->ids, d_list, m, species, e->species, (Rec<3>*)e->pos[e->cur],
                                                                    e->verlet ? e->qpos[e->cur] : nullptr);
    note_launch();
    GBMD_CUDA_TRY(cudaFreeAsync(d_list, e->st));
    // lists are built with per-pair radii: rebuild before the next step
    uint32_t one = 1;
    GBMD_CUDA_TRY(cudaMemcpyAsync(e->ctl, &one, 4, cudaMemcpyHostToDevice, e->st));
    if (e->sys.pinned) { // the moving set (the thermostat's zero-momentum ranks) may have changed
        std::vector<uint32_t> sp(e->n);
        GBMD_TRY(gbmd_read_state(e, nullptr, nullptr, sp.data()));
        GBMD_TRY(upload_ranks(e, sp.data()));
    }
    return gbmd_sync(e);
}

int gbmd_set_species_velocity(gbmd_engine* e, uint32_t species, const double* v) {
    if (!e || !v) return fail(GBMD_E_INVALID, "null argument");
    if (species >= e->sys.nspecies) return fail(GBMD_E_INVALID, "species index out of range");
    int3 d = make_int3(to_step_displacement(e->sys, v[0]), to_step_displacement(e->sys, v[1]), e->D == 3 ? to_step_displacement(e->sys, v[2]) : 0);
    k_set_species_velocity<<<blocks_for(e->n, 256), 256, 0, e->st>>>(e->n, (uint32_t)e->D, e->species, species, d, e->vel);
    note_launch();
    GBMD_CUDA_TRY(cudaGetLastError());
    return GBMD_OK;
}

int gbmd_sort_now(gbmd_engine* e) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    GBMD_TRY(prepare_pairs(e));
    return gbmd_sync(e);
}

int gbmd_set_bonds(gbmd_engine* e, const gbmd_bond_type* types, uint32_t ntypes, const uint32_t* bonds, uint32_t nbonds) {
    if (!e || (ntypes && !types) || (nbonds && !bonds)) return fail(GBMD_E_INVALID, "null argument");
    if (e->D != 2 && nbonds) return fail(GBMD_E_UNSUPPORTED, "bonds are two-dimensional (IntEngine; IntEngine3 has none)");
    if (e->opt.arith != GBMD_ARITH_F32 && nbonds) return fail(GBMD_E_UNSUPPORTED, "integer table forces take plain pair systems only");
    if (ntypes > GBMD_MAX_BOND_TYPES) return fail(GBMD_E_INVALID, "at most GBMD_MAX_BOND_TYPES bond types");
    for (uint32_t t = 0; t < ntypes; t++) {
        const gbmd_bond_type& b = types[t];
        if ((b.kind != GBMD_BOND_HARMONIC && b.kind != GBMD_BOND_FENE) || !(std::fabs(b.k) < INFINITY) || !(b.r0 >= 0.0 && b.r0 < INFINITY) ||
            (b.kind == GBMD_BOND_FENE && !(b.r0 > 0.0)))
            return fail(GBMD_E_INVALID, "a bond type is harmonic or FENE with finite k and r0 >= 0 (FENE: r0 > 0)");
    }
    std::vector<uint32_t> tab;
    if (nbonds) {
        tab.assign((size_t)e->n * 8, 0xffffffffu);
        std::vector<uint32_t> used(e->n, 0);
        for (uint32_t q = 0; q < nbonds; q++) {
            const uint32_t a = bonds[3 * q], b = bonds[3 * q + 1], t = bonds[3 * q + 2];
            if (a >= e->n || b >= e->n || a == b || t >= ntypes) return fail(GBMD_E_INVALID, "a bond joins two particles (ids < n) with a known type");
            for (int end = 0; end < 2; end++) { // System::partner_table (system.rs:311-324)
                const uint32_t me = end ? b : a, other = end ? a : b;
                if (used[me] >= GBMD_MAX_BONDS) return fail(GBMD_E_INVALID, "at most GBMD_MAX_BONDS bonds per particle");
                tab[(size_t)me * 8 + 2 * used[me]] = other;
                tab[(size_t)me * 8 + 2 * used[me] + 1] = t;
                used[me]++;
            }
        }
    }
    GBMD_CUDA_TRY(cudaStreamSynchronize(e->st));
    if (nbonds && !e->bond_tab) {
        GBMD_TRY(allocT(e, &e->bond_tab, (size_t)e->n * 8));
        GBMD_TRY(allocT(e, &e->slot_of, (size_t)e->n));
    }
    if (nbonds) {
        GBMD_CUDA_TRY(cudaMemcpyAsync(e->bond_tab, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice, e->st));
        k_slot_of<<<blocks_for(e->n, 256), 256, 0, e->st>>>(e->n, e->ids, e->slot_of); // (list builds keep it after)
        note_launch();
    }
    e->P.bonds = nbonds ? 1u : 0u;
    e->P.bond_tab = e->bond_tab;
    e->bond_types_h.assign(types, types + ntypes);
    e->bonds_h.clear();
    for (uint32_t q = 0; q < nbonds; q++) e->bonds_h.push_back({bonds[3 * q], bonds[3 * q + 1], bonds[3 * q + 2]});
    e->P.slot_of = e->slot_of;
    for (uint32_t t = 0; t < 4; t++) {
        e->P.bond_fene[t] = t < ntypes && types[t].kind == GBMD_BOND_FENE;
        e->P.bond_k[t] = t < ntypes ? (float)types[t].k : 0.0f;
        e->P.bond_r0[t] = t < ntypes ? (float)types[t].r0 : 0.0f;
    }
    // graphs hold the old parameter block by value: capture again on the next step
    for (int p = 0; p < 2; p++)
        for (int b = 0; b < 5; b++)
            if (e->exec[p][b]) {
                GBMD_CUDA_TRY(cudaGraphExecDestroy(e->exec[p][b]));
                e->exec[p][b] = nullptr;
            }
    GBMD_TRY(setup_step_loop(e));
    return gbmd_sync(e);
}

int gbmd_set_piston(gbmd_engine* e, const gbmd_piston* p) {
    if (!e || !p) return fail(GBMD_E_INVALID, "null argument");
    if (p->drive == GBMD_PISTON_NONE) {
        GBMD_CUDA_TRY(cudaStreamSynchronize(e->st));
        e->P.piston_drive = 0;
    } else {
        if (e->D != 2) return fail(GBMD_E_UNSUPPORTED, "pistons are two-dimensional (IntEngine; IntEngine3 has none)");
        if ((e->P.periodic >> 1) & 1u) return fail(GBMD_E_INVALID, "a piston needs walls on y");
        const double top = (double)e->sys.box_len[1] * (1.0 / 4294967296.0);
        const bool finite = std::isfinite(p->speed) && std::isfinite(p->mass) && std::isfinite(p->force) && std::isfinite(p->start) &&
                            std::isfinite(p->min);
        if (p->drive > GBMD_PISTON_FREE || !finite || !(p->min < p->start && p->start <= top) || (p->drive == GBMD_PISTON_FREE && !(p->mass > 0.0)))
            return fail(GBMD_E_INVALID, "a piston is driven at a speed or free (mass > 0), with min < start <= the box height");
        GBMD_CUDA_TRY(cudaStreamSynchronize(e->st));
        if (!e->piston) GBMD_TRY(allocT(e, &e->piston, 1));
        PistonState ps{};
        ps.w = sat_i64_host(std::round(p->start * 4294967296.0)); // fixed::to_fixed (fixed.rs:21-23)
        ps.v = p->drive == GBMD_PISTON_SPEED ? to_step_displacement(e->sys, p->speed) : 0;
        GBMD_CUDA_TRY(cudaMemcpyAsync(e->piston, &ps, sizeof(ps), cudaMemcpyHostToDevice, e->st));
        e->P.piston_drive = p->drive;
        e->P.piston_mass = p->mass;
        e->P.piston_ext = p->force;
        e->P.piston_lo = sat_i64_host(std::round(p->min * 4294967296.0));
        e->P.piston_hi = sat_i64_host(std::round(top * 4294967296.0));
        e->P.piston = e->piston;
    }
    // graphs hold the old parameter block by value: capture again on the next step
    for (int q = 0; q < 2; q++)
        for (int b = 0; b < 5; b++)
            if (e->exec[q][b]) {
                GBMD_CUDA_TRY(cudaGraphExecDestroy(e->exec[q][b]));
                e->exec[q][b] = nullptr;
            }
    GBMD_TRY(setup_step_loop(e));
    return gbmd_sync(e);
}

int gbmd_read_piston(gbmd_engine* e, int64_t* height, int32_t* velocity, double* work, double* force) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    PistonState ps{};
    if (e->P.piston_drive) {
        GBMD_CUDA_TRY(cudaMemcpyAsync(&ps, e->piston, sizeof(ps), cudaMemcpyDeviceToHost, e->st));
        GBMD_CUDA_TRY(cudaStreamSynchronize(e->st));
    }
    if (height) *height = ps.w;
    if (velocity) *velocity = ps.v;
    if (work) *work = ps.work;
    if (force) *force = ps.gas;
    return GBMD_OK;
}

int gbmd_set_piston_speed(gbmd_engine* e, double speed) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    if (!e->P.piston_drive) return fail(GBMD_E_INVALID, "the engine has no piston");
    if (!std::isfinite(speed)) return fail(GBMD_E_INVALID, "a finite speed");
    const int32_t v = to_step_displacement(e->sys, speed);
    GBMD_CUDA_TRY(cudaMemcpyAsync((char*)e->piston + offsetof(PistonState, v), &v, 4, cudaMemcpyHostToDevice, e->st));
    return gbmd_sync(e);
}

// The partner-table rows of these ids from the bond list (System::partner_table, system.rs:
// 311-324: each bond appended to both ends' rows in list order), uploaded.
static int upload_partner_rows(gbmd_engine* e, std::initializer_list<uint32_t> ids) {
    for (uint32_t id : ids) {
        uint32_t row[8];
        std::fill(row, row + 8, 0xffffffffu);
        uint32_t used = 0;
        for (const auto& b : e->bonds_h)
            for (int end = 0; end < 2; end++)
                if (b[end] == id && used < GBMD_MAX_BONDS) {
                    row[2 * used] = b[1 - end];
                    row[2 * used + 1] = b[2];
                    used++;
                }
        GBMD_CUDA_TRY(cudaMemcpyAsync(e->bond_tab + 8 * (size_t)id, row, sizeof(row), cudaMemcpyHostToDevice, e->st));
    }
    return gbmd_sync(e);
}

int gbmd_remove_bond(gbmd_engine* e, uint32_t a, uint32_t b, int32_t* removed) {
    if (!e || !removed) return fail(GBMD_E_INVALID, "null argument");
    *removed = 0;
    const size_t before = e->bonds_h.size();
    e->bonds_h.erase(std::remove_if(e->bonds_h.begin(), e->bonds_h.end(),
                                    [&](const std::array<uint32_t, 3>& x) { return (x[0] == a && x[1] == b) || (x[0] == b && x[1] == a); }),
                     e->bonds_h.end());
    if (e->bonds_h.size() == before) return GBMD_OK;
    *removed = 1;
    return upload_partner_rows(e, {a, b});
}

int gbmd_add_bond(gbmd_engine* e, uint32_t a, uint32_t b, uint32_t type, int32_t* added) {
    if (!e || !added) return fail(GBMD_E_INVALID, "null argument");
    *added = 0;
    if (e->D != 2) return fail(GBMD_E_UNSUPPORTED, "bonds are two-dimensional (IntEngine; IntEngine3 has none)");
    if (type >= e->bond_types_h.size()) return fail(GBMD_E_INVALID, "add_bond needs a system built with that bond type (gbmd_set_bonds)");
    if (a >= e->n || b >= e->n) return fail(GBMD_E_INVALID, "particle ids < n");
    auto count = [&](uint32_t id) {
        uint32_t c = 0;
        for (const auto& x : e->bonds_h) c += (x[0] == id) + (x[1] == id);
        return c;
    };
    for (const auto& x : e->bonds_h)
        if ((x[0] == a && x[1] == b) || (x[0] == b && x[1] == a)) return GBMD_OK; // already bonded
    if (a == b || count(a) >= GBMD_MAX_BONDS || count(b) >= GBMD_MAX_BONDS) return GBMD_OK;
    e->bonds_h.push_back({a, b, type});
    if (!e->P.bonds) { // the first bond: the table, and graphs that take the bond pass
        std::vector<uint32_t> flat;
        for (const auto& x : e->bonds_h) flat.insert(flat.end(), x.begin(), x.end());
        std::vector<gbmd_bond_type> types = e->bond_types_h;
        GBMD_TRY(gbmd_set_bonds(e, types.data(), (uint32_t)types.size(), flat.data(), (uint32_t)e->bonds_h.size()));
    } else {
        GBMD_TRY(upload_partner_rows(e, {a, b}));
    }
    *added = 1;
    return GBMD_OK;
}

int gbmd_flip_species_bit(gbmd_engine* e, uint32_t species_mask, uint32_t axis, uint32_t bit) {
    if (!e || axis >= (uint32_t)e->D || bit > 62) return fail(GBMD_E_INVALID, "bad flip_species_bit argument");
    GBMD_TRY(prepare_pairs(e)); // wraps the positions into the box (they drift out between list builds)
    if (e->D == 2) k_flip_species<2><<<blocks_for(e->n, 256), 256, 0, e->st>>>(e->n, e->species, species_mask, axis, bit, (Rec<2>*)e->pos[e->cur]);
    else k_flip_species<3><<<blocks_for(e->n, 256), 256, 0, e->st>>>(e->n, e->species, species_mask, axis, bit, (Rec<3>*)e->pos[e->cur]);
    note_launch();
    uint32_t one = 1;
    GBMD_CUDA_TRY(cudaMemcpyAsync(e->ctl, &one, 4, cudaMemcpyHostToDevice, e->st));
    return gbmd_sync(e);
}

int gbmd_update_system(gbmd_engine* e, const gbmd_system* sys) {
    if (!e || !sys) return fail(GBMD_E_INVALID, "null argument");
    GBMD_TRY(validate_system(*sys, e->n));
    if (e->P.piston_drive && ((sys->periodic >> 1) & 1u))
        return fail(GBMD_E_INVALID, "the engine has a piston: y keeps its walls");
    const gbmd_system& o = e->sys;
    if (sys->dim != o.dim || sys->nspecies != o.nspecies) return fail(GBMD_E_INVALID, "update_system keeps the dimension and the species count");
    for (uint32_t a = 0; a < o.dim; a++)
        if (sys->box_len[a] != o.box_len[a]) return fail(GBMD_E_INVALID, "update_system keeps the box");
    if (rc_max(*sys) > rc_max(o) + 1e-12) return fail(GBMD_E_INVALID, "cutoffs cannot grow at run time");
    if (e->P.int_mode) {
        bool same = sys->dt == o.dt && sys->pinned == o.pinned;
        for (uint32_t k = 0; k < o.nspecies; k++) same = same && sys->masses[k] == o.masses[k];
        for (uint32_t k = 0; k < o.nspecies * o.nspecies; k++)
            same = same && std::memcmp(&sys->pairs[k], &o.pairs[k], sizeof(gbmd_pair)) == 0;
        if (!same) return fail(GBMD_E_INVALID, "integer tables are fixed at creation: pairs, masses, dt and pinned species cannot change");
    }
    GBMD_TRY(gbmd_sync(e));
    const bool pinned_changed = sys->pinned != o.pinned;
    Params old = e->P;
    e->sys = *sys;
    fill_params(e->P, e->sys, e->n, e->skin, old.cap, old.nc);
    if (e->opt.flags & GBMD_FLAG_NO_PATH_BOUND) e->P.ub_thr = 0;
    // the geometry and list sizing of creation, the integer tables, the slabs
    e->P.key_shift = old.key_shift;
    e->P.sub_scale = old.sub_scale;
    e->P.sub_delta = old.sub_delta;
    e->P.int_mode = old.int_mode;
    e->P.itab_len = old.itab_len;
    e->P.itab = old.itab;
    e->P.ipair = old.ipair;
    std::memcpy(e->P.irc2, old.irc2, sizeof(old.irc2));
    // the half-shell windows and the bonds (set apart from the System)
    e->P.half_lists = old.half_lists;
    e->P.win_cap = old.win_cap;
    e->P.bonds = old.bonds;
    std::memcpy(e->P.bond_fene, old.bond_fene, sizeof(old.bond_fene));
    std::memcpy(e->P.bond_k, old.bond_k, sizeof(old.bond_k));
    std::memcpy(e->P.bond_r0, old.bond_r0, sizeof(old.bond_r0));
    e->P.bond_tab = old.bond_tab;
    e->P.slot_of = old.slot_of;
    e->P.ids_list = old.ids_list;
    e->P.ledger = old.ledger;
    e->P.ledger_per_wall = old.ledger_per_wall;
    e->P.clock_word = old.clock_word;
    e->P.piston_drive = old.piston_drive; // and the piston
    e->P.piston_mass = old.piston_mass;
    e->P.piston_ext = old.piston_ext;
    e->P.piston_lo = old.piston_lo;
    e->P.piston_hi = old.piston_hi;
    e->P.piston = old.piston;
    // graphs hold the old parameter block by value: capture again on the next step
    for (int p = 0; p < 2; p++)
        for (int b = 0; b < 5; b++)
            if (e->exec[p][b]) {
                GBMD_CUDA_TRY(cudaGraphExecDestroy(e->exec[p][b]));
                e->exec[p][b] = nullptr;
            }
    GBMD_TRY(setup_step_loop(e));
    uint32_t one = 1;
    GBMD_CUDA_TRY(cudaMemcpyAsync(e->ctl, &one, 4, cudaMemcpyHostToDevice, e->st));
    if (pinned_changed) {
        std::vector<uint32_t> sp(e->n);
        GBMD_TRY(gbmd_read_state(e, nullptr, nullptr, sp.data()));
        GBMD_TRY(upload_ranks(e, sp.data()));
    }
    return gbmd_sync(e);
}

int gbmd_energy(gbmd_engine* e, double* kinetic, double* potential) {
    gbmd_frame f;
    GBMD_TRY(gbmd_observe(e, &f, nullptr, 0, 0.0, nullptr, 0, 0));
    if (kinetic) *kinetic = f.kinetic;
    if (potential) *potential = f.potential;
    return GBMD_OK;
}

int gbmd_list_stats(gbmd_engine* e, uint32_t* rebuilds, int32_t* overflow) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    uint32_t c[11];
    GBMD_CUDA_TRY(cudaMemcpyAsync(c, e->ctl, sizeof(c), cudaMemcpyDeviceToHost, e->st));
    GBMD_CUDA_TRY(cudaStreamSynchronize(e->st));
    e->loop_iters = c[CTL_LOOP_ITERS];
    if (rebuilds) *rebuilds = c[2];
    if (overflow) *overflow = c[1] ? 1 : 0;
    return GBMD_OK;
}

int gbmd_state_hash(gbmd_engine* e, uint64_t* hash) {
    if (!e || !hash) return fail(GBMD_E_INVALID, "null argument");
    size_t n = e->n, D = e->D;
    std::vector<int64_t> pos(n * D);
    std::vector<int32_t> vel(n * D);
    std::vector<uint32_t> sp(n);
    GBMD_TRY(gbmd_read_state(e, pos.data(), vel.data(), sp.data()));
    *hash = gbmd_hash_state((uint32_t)D, pos.data(), vel.data(), sp.data(), (uint32_t)n);
    return GBMD_OK;
}

int gbmd_read_compartment_ledger(gbmd_engine* e, uint32_t cap, double* energy, double* impulse, uint64_t* hits, uint32_t* per_wall) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    const uint32_t pw = e->P.ledger_per_wall;
    if (per_wall) *per_wall = pw;
    if (!energy && !impulse && !hits) return GBMD_OK;
    if (cap < pw) return fail(GBMD_E_INVALID, "room for fewer compartments per wall than the engine keeps");
    std::vector<unsigned long long> l(3 * (size_t)GBMD_LEDGER_SLOTS * pw);
    GBMD_CUDA_TRY(cudaMemcpyAsync(l.data(), e->ledger, l.size() * 8, cudaMemcpyDeviceToHost, e->st));
    GBMD_CUDA_TRY(cudaStreamSynchronize(e->st));
    for (int w = 0; w < GBMD_LEDGER_SLOTS; w++)
        for (uint32_t c = 0; c < cap; c++) {
            const size_t q = (size_t)w * cap + c, at = 3 * ((size_t)w * pw + c);
            const bool in = c < pw;
            if (energy) energy[q] = in ? (double)(long long)l[at] * (1.0 / 16777216.0) : 0.0;
            if (hits) hits[q] = in ? (uint64_t)l[at + 1] : 0;
            if (impulse) impulse[q] = in ? (double)(long long)l[at + 2] * (1.0 / 16777216.0) : 0.0;
        }
    return GBMD_OK;
}

int gbmd_read_ledger(gbmd_engine* e, double* energy, double* impulse, uint64_t* hits) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    const uint32_t pw = e->P.ledger_per_wall;
    std::vector<unsigned long long> l(3 * (size_t)GBMD_LEDGER_SLOTS * pw);
    GBMD_CUDA_TRY(cudaMemcpyAsync(l.data(), e->ledger, l.size() * 8, cudaMemcpyDeviceToHost, e->st));
    GBMD_CUDA_TRY(cudaStreamSynchronize(e->st));
    for (int w = 0; w < GBMD_LEDGER_SLOTS; w++) { // CompartmentLedger::totals (walls.rs:63-71), in integers
        unsigned long long t[3] = {0, 0, 0};
        for (uint32_t c = 0; c < pw; c++)
            for (int q = 0; q < 3; q++) t[q] += l[3 * ((size_t)w * pw + c) + q];
        if (energy) energy[w] = (double)(long long)t[0] * (1.0 / 16777216.0);
        if (hits) hits[w] = (uint64_t)t[1];
        if (impulse) impulse[w] = (double)(long long)t[2] * (1.0 / 16777216.0);
    }
    return GBMD_OK;
}

int gbmd_counters(gbmd_engine* e, int64_t* steps, uint32_t* clock) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    if (steps) *steps = e->steps;
    if (clock) *clock = e->clock;
    return GBMD_OK;
}

int gbmd_stream(gbmd_engine* e, void** stream) {
    if (!e || !stream) return fail(GBMD_E_INVALID, "null argument");
    *stream = (void*)e->st;
    return GBMD_OK;
}

int gbmd_launch_count(gbmd_engine* e, uint64_t* launches) {
    if (!e || !launches) return fail(GBMD_E_INVALID, "null argument");
    uint32_t rebuilds = 0;
    int32_t ov = 0;
    GBMD_TRY(gbmd_list_stats(e, &rebuilds, &ov));
    *launches = e->launches + (uint64_t)rebuilds * e->body_launches + 3ull * e->loop_iters;
    return GBMD_OK;
}

int gbmd_time_phases(gbmd_engine* e, uint32_t steps, double* force_ms, double* rebuild_ms, uint32_t* rebuilds) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    GBMD_TRY(gbmd_sync(e));
    cudaEvent_t a, b, c;
    GBMD_CUDA_TRY(cudaEventCreate(&a));
    GBMD_CUDA_TRY(cudaEventCreate(&b));
    GBMD_CUDA_TRY(cudaEventCreate(&c));
    double tf = 0.0, tr = 0.0;
    uint32_t nr = 0;
    for (uint32_t k = 0; k < steps; k++) {
        uint32_t flag = 0;
        if (e->verlet) {
            GBMD_CUDA_TRY(cudaMemcpyAsync(&flag, e->ctl, 4, cudaMemcpyDeviceToHost, e->st));
            GBMD_CUDA_TRY(cudaStreamSynchronize(e->st));
        }
        GBMD_CUDA_TRY(cudaEventRecord(a, e->st));
        if (flag) {
            enqueue_rebuild(e, e->st);
            nr++;
        }
        GBMD_CUDA_TRY(cudaEventRecord(b, e->st));
        enqueue_force(e, e->st);
        GBMD_CUDA_TRY(cudaEventRecord(c, e->st));
        GBMD_CUDA_TRY(cudaEventSynchronize(c));
        float m1 = 0.f, m2 = 0.f;
        cudaEventElapsedTime(&m1, a, b);
        cudaEventElapsedTime(&m2, b, c);
        if (flag) tr += m1;
        tf += m2;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaEventDestroy(c);
    e->steps += steps;
    e->clock += steps;
    e->tcount += steps;
    if (force_ms) *force_ms = steps ? tf / steps : 0.0;
    if (rebuild_ms) *rebuild_ms = nr ? tr / nr : 0.0;
    if (rebuilds) *rebuilds = nr;
    return check_ctl(e);
}

int gbmd_time_thermostat(gbmd_engine* e, uint32_t reps, double* ms) {
    if (!e || !ms) return fail(GBMD_E_INVALID, "null argument");
    if (!e->opt.rescale_every) return fail(GBMD_E_INVALID, "the engine has no velocity-rescale thermostat");
    GBMD_TRY(gbmd_sync(e));
    cudaEvent_t a, b;
    GBMD_CUDA_TRY(cudaEventCreate(&a));
    GBMD_CUDA_TRY(cudaEventCreate(&b));
    double total = 0.0;
    for (uint32_t k = 0; k < reps; k++) {
        GBMD_CUDA_TRY(cudaEventRecord(a, e->st));
        enqueue_thermo(e, e->st);
        GBMD_CUDA_TRY(cudaEventRecord(b, e->st));
        GBMD_CUDA_TRY(cudaEventSynchronize(b));
        float m = 0.0f;
        cudaEventElapsedTime(&m, a, b);
        total += m;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms = reps ? total / reps : 0.0;
    return check_ctl(e);
}

int gbmd_time_loop(gbmd_engine* e, uint32_t steps, uint32_t* taken, double* ms_per_step, uint32_t* launches) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    if (!e->loop_lanes) return fail(GBMD_E_UNSUPPORTED, "this engine does not step through the persistent loop");
    GBMD_TRY(gbmd_sync(e));
    cudaEvent_t a, b;
    GBMD_CUDA_TRY(cudaEventCreate(&a));
    GBMD_CUDA_TRY(cudaEventCreate(&b));
    uint32_t total = 0, nl = 0;
    double t = 0.0;
    int rc = GBMD_OK;
    while (total < steps) {
        uint32_t c[16];
        GBMD_CUDA_TRY(cudaMemcpyAsync(c, e->ctl, sizeof(c), cudaMemcpyDeviceToHost, e->st));
        GBMD_CUDA_TRY(cudaStreamSynchronize(e->st));
        if (c[0]) enqueue_rebuild(e, e->st);
        k_loop_begin<<<1, 1, 0, e->st>>>(e->ctl);
        note_launch();
        GBMD_CUDA_TRY(cudaEventRecord(a, e->st));
        GBMD_CUDA_TRY(enqueue_loop(e, e->st));
        GBMD_CUDA_TRY(cudaEventRecord(b, e->st));
        GBMD_CUDA_TRY(cudaEventSynchronize(b));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        GBMD_CUDA_TRY(cudaMemcpyAsync(c, e->ctl, sizeof(c), cudaMemcpyDeviceToHost, e->st));
        GBMD_CUDA_TRY(cudaStreamSynchronize(e->st));
        t += ms;
        nl++;
        total += c[CTL_LOOP_DONE];
        if (c[CTL_LOOP_ERR] || c[CTL_LOOP_DONE] == 0) {
            rc = check_ctl(e);
            if (rc == GBMD_OK) rc = fail(GBMD_E_TIMEOUT, "the persistent loop took no step");
            break;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    e->steps += total;
    e->clock += total;
    e->tcount += total;
    if (taken) *taken = total;
    if (ms_per_step) *ms_per_step = total ? t / total : 0.0;
    if (launches) *launches = nl;
    if (rc != GBMD_OK) return rc;
    return check_ctl(e);
}

int gbmd_debug_bin(gbmd_engine* e, const uint32_t* cells, uint32_t* keys, uint32_t* start, uint32_t* items, uint32_t* order) {
    if (!e || !cells) return fail(GBMD_E_INVALID, "null argument");
    Params P = e->P;
    uint64_t ncell = 1;
    for (int a = 0; a < e->D; a++) {
        if (cells[a] < 1) return fail(GBMD_E_INVALID, "cells must be positive");
        ncell *= cells[a];
        if (ncell >= UINT32_MAX) return fail(GBMD_E_INVALID, "too many cells");
    }
    set_cells(P, cells, (uint32_t)e->D);
    uint32_t* st2 = nullptr;
    GBMD_CUDA_TRY(cudaMalloc(&st2, ((size_t)P.ncell + 1) * 4));
    uint32_t* saved = e->start;
    e->start = st2;
    uint32_t n = e->n;
    std::vector<uint32_t> k(n);
    // keys in storage order first (before the sort overwrites them)
    if (e->D == 2) k_keys<2><<<blocks_for(n, 256), 256, 0, e->st>>>(P, (const Rec<2>*)e->pos[e->cur], e->keys[0], e->vals[0]);
    else k_keys<3><<<blocks_for(n, 256), 256, 0, e->st>>>(P, (const Rec<3>*)e->pos[e->cur], e->keys[0], e->vals[0]);
    cudaMemcpyAsync(k.data(), e->keys[0], (size_t)n * 4, cudaMemcpyDeviceToHost, e->st);
    if (order) cudaMemcpyAsync(order, e->ids, (size_t)n * 4, cudaMemcpyDeviceToHost, e->st);
    if (e->D == 2) enqueue_bin<2>(e, e->st, P);
    else enqueue_bin<3>(e, e->st, P);
    if (start) cudaMemcpyAsync(start, e->start, ((size_t)P.ncell + 1) * 4, cudaMemcpyDeviceToHost, e->st);
    if (items) cudaMemcpyAsync(items, e->vals[e->sorted], (size_t)n * 4, cudaMemcpyDeviceToHost, e->st);
    cudaError_t err = cudaStreamSynchronize(e->st);
    e->start = saved;
    cudaFree(st2);
    if (err != cudaSuccess) return fail(GBMD_E_CUDA, cudaGetErrorString(err));
    if (keys) std::memcpy(keys, k.data(), (size_t)n * 4);
    // the sort state is scratch only: the pair structure must be rebuilt before the next use
    uint32_t one = 1;
    GBMD_CUDA_TRY(cudaMemcpyAsync(e->ctl, &one, 4, cudaMemcpyHostToDevice, e->st));
    return gbmd_sync(e);
}

int gbmd_debug_barrier_timeout(gbmd_engine* e, uint32_t blocks) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    if (blocks < 2 || blocks > 64) return fail(GBMD_E_INVALID, "blocks must be 2 .. 64");
    GBMD_TRY(gbmd_sync(e));
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(128);
    cfg.stream = e->st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    GBMD_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_barrier_absent, e->ctl, 0u));
    note_launch();
    return gbmd_sync(e);
}

int gbmd_debug_list(gbmd_engine* e, uint32_t* counts, uint32_t* nbr, uint64_t nbr_cap) {
    if (!e || !counts || !nbr) return fail(GBMD_E_INVALID, "null argument");
    if (!e->verlet) return fail(GBMD_E_INVALID, "the engine has no Verlet list (cell mode)");
    GBMD_TRY(prepare_pairs(e));
    GBMD_TRY(gbmd_sync(e));
    size_t n = e->n, cap4 = ((size_t)e->P.cap + 3) & ~(size_t)3;
    size_t total = (n + 31) / 32 * 32 * cap4;
    std::vector<uint32_t> cnt(n), ids(n), lst(total);
    GBMD_CUDA_TRY(cudaMemcpy(cnt.data(), e->nbr_count, n * 4, cudaMemcpyDeviceToHost));
    GBMD_CUDA_TRY(cudaMemcpy(ids.data(), e->ids, n * 4, cudaMemcpyDeviceToHost));
    GBMD_CUDA_TRY(cudaMemcpy(lst.data(), e->nbr, total * 4, cudaMemcpyDeviceToHost));
    auto slot = [&](size_t i, size_t k) { return ((i >> 5) * cap4 + (k & ~(size_t)3)) * 32 + ((i & 31) << 2) + (k & 3); };
    std::vector<uint32_t> slot_of(n);
    for (size_t s = 0; s < n; s++) slot_of[ids[s]] = (uint32_t)s;
    if (e->half) {
        // Half-shell lists hold each pair once, by window and offset in the neighbour's row:
        // decode them to slots and return both ends' sets, as a full list would hold them.
        const uint32_t nx = e->P.nc[0], ny = e->P.nc[1], nz = e->P.nc[2];
        std::vector<uint32_t> keys((size_t)n), start((size_t)e->P.ncell + 1);
        GBMD_CUDA_TRY(cudaMemcpy(keys.data(), e->keys[e->sorted], n * 4, cudaMemcpyDeviceToHost));
        GBMD_CUDA_TRY(cudaMemcpy(start.data(), e->start, start.size() * 4, cudaMemcpyDeviceToHost));
        std::vector<std::vector<uint32_t>> sets(n);
        for (size_t s = 0; s < n; s++) {
            const uint32_t row = keys[s] / nx, y = row % ny, z = row / ny;
            for (size_t q = 0; q < cnt[s]; q++) {
                const uint32_t ent = lst[slot(s, q)], w = (ent >> HALF_WIN_SHIFT) & 15u;
                if (w >= HALF_WINDOWS) return fail(GBMD_E_INVALID, "corrupt half-shell list entry");
                const uint32_t j = start[(size_t)half_window_row(ny, nz, y, z, w) * nx] + (ent & HALF_OFF_MASK);
                if (j >= n) return fail(GBMD_E_INVALID, "corrupt half-shell list entry");
                sets[ids[s]].push_back(ids[j]);
                sets[ids[j]].push_back(ids[s]);
            }
        }
        uint64_t off = 0;
        for (size_t id = 0; id < n; id++) {
            counts[id] = (uint32_t)sets[id].size();
            if (off + sets[id].size() > nbr_cap) return fail(GBMD_E_INVALID, "nbr_cap too small");
            for (uint32_t j : sets[id]) nbr[off++] = j;
        }
        return GBMD_OK;
    }
    uint64_t off = 0;
    for (size_t id = 0; id < n; id++) {
        size_t s = slot_of[id];
        counts[id] = cnt[s];
        if (off + cnt[s] > nbr_cap) return fail(GBMD_E_INVALID, "nbr_cap too small");
        for (size_t q = 0; q < cnt[s]; q++) nbr[off++] = ids[lst[slot(s, q)] & ((1u << 26) - 1u)];
    }
    return GBMD_OK;
}

const char* gbmd_last_error(void) { return t_error.c_str(); }
const char* gbmd_version(void) { return "gbmd 0.1 (sm_103a)"; }

} // extern "C"

// ------------------------------------------------------------------ observables
namespace {

// RDF pair counts over unordered pairs of the cell-sorted scratch state (cells of side >= rmax,
// at least three per axis). A candidate j of neighbour cell cj sits at d = relf[j] + base with
// base = (cj - c) cell_w + image - (xi - c cell_w), an exact integer converted once per cell, so
// the candidate costs one 16-byte load and a few f32 operations. The f32 estimate of
// r bins / rmax is within `margin` bins of the exact value (the host bounds the conversions'
// and the sum's rounding); a pair clear of every bin edge by that much, or beyond `lim2f`, is
// decided by it, the rest (a fraction ~2 margin of the pairs) by the f64 definition on the exact
// integer separation.
template <int D>
__global__ void __launch_bounds__(128) k_rdf(Params P, const Rec<D>* pos, const float4* relf, const uint32_t* keys, const uint32_t* start,
                                             uint32_t bins, double scale, float scalef, float lim2f, float margin, unsigned long long* out) {
    extern __shared__ uint32_t h[];
    for (uint32_t b = threadIdx.x; b < bins; b += blockDim.x) h[b] = 0;
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P.n) {
        int64_t xi[3], reli[3];
        load_particle<D, false>(pos, nullptr, i, xi);
        uint32_t c[3];
        cell_coords(P, keys[i], c);
#pragma unroll
        for (int a = 0; a < 3; a++) reli[a] = a < D ? xi[a] - (int64_t)c[a] * P.cell_w[a] : 0;
        const float top = (float)bins - margin, hi = 1.0f - margin;
        for (int oz = 0; oz < (D == 3 ? 3 : 1); oz++) {
            int64_t z = D == 3 ? (int64_t)c[2] + oz - 1 : 0, sz = 0;
            if (D == 3 && z < 0) z += P.nc[2], sz = image_shift(P, 2, -P.box[2]);
            if (D == 3 && z >= (int64_t)P.nc[2]) z -= P.nc[2], sz = image_shift(P, 2, P.box[2]);
            for (int oy = 0; oy < 3; oy++) {
                int64_t y = (int64_t)c[1] + oy - 1, sy = 0;
                if (y < 0) y += P.nc[1], sy = image_shift(P, 1, -P.box[1]);
                if (y >= (int64_t)P.nc[1]) y -= P.nc[1], sy = image_shift(P, 1, P.box[1]);
                for (int ox = 0; ox < 3; ox++) {
                    int64_t x = (int64_t)c[0] + ox - 1, sx = 0;
                    if (x < 0) x += P.nc[0], sx = image_shift(P, 0, -P.box[0]);
                    if (x >= (int64_t)P.nc[0]) x -= P.nc[0], sx = image_shift(P, 0, P.box[0]);
                    const uint32_t cell = (uint32_t)((z * P.nc[1] + y) * P.nc[0] + x);
                    const uint32_t j0 = max(start[cell], i + 1), j1 = start[cell + 1];
                    if (j0 >= j1) continue;
                    const float b0 = off_f32((x - (int64_t)c[0]) * P.cell_w[0] + sx - reli[0]);
                    const float b1 = off_f32((y - (int64_t)c[1]) * P.cell_w[1] + sy - reli[1]);
                    const float b2 = D == 3 ? off_f32((z - (int64_t)c[2]) * P.cell_w[2] + sz - reli[2]) : 0.0f;
#pragma unroll 2
                    for (uint32_t j = j0; j < j1; j++) {
                        const float4 r = relf[j];
                        const float d0 = __fadd_rn(r.x, b0), d1 = __fadd_rn(r.y, b1);
                        float r2f = __fmaf_rn(d1, d1, __fmul_rn(d0, d0));
                        if (D == 3) {
                            const float d2 = __fadd_rn(r.z, b2);
                            r2f = __fmaf_rn(d2, d2, r2f);
                        }
                        if (r2f > lim2f) continue;
                        const float rf = __fmul_rn(__fsqrt_rn(r2f), scalef);
                        const float fl = floorf(rf), fr = __fsub_rn(rf, fl);
                        int k;
                        if (fr > margin && fr < hi && rf < top) {
                            k = (int)fl;
                        } else {
                            int64_t xj[3], d[3];
                            load_particle<D, false>(pos, nullptr, j, xj);
#pragma unroll
                            for (int a = 0; a < D; a++) d[a] = min_image(xj[a] - xi[a], P.box[a], P.half[a]);
                            k = rdf_bin_exact<D>(d, bins, scale);
                        }
                        if (k >= 0) atomicAdd(&h[k], 1u);
                    }
                }
            }
        }
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < bins; b += blockDim.x)
        if (h[b]) atomicAdd(out + b, (unsigned long long)h[b]);
}

// The same counts for cells wider than the f32 offsets of the scratch state cover (rmax beyond
// about 40 sigma): every candidate from the exact integer separation.
template <int D>
__global__ void k_rdf_wide(Params P, const Rec<D>* pos, const uint32_t* keys, const uint32_t* start, uint32_t bins, double scale,
                      float scalef, float lim2f, float margin, unsigned long long* out) {
    extern __shared__ uint32_t h[];
    for (uint32_t b = threadIdx.x; b < bins; b += blockDim.x) h[b] = 0;
    __syncthreads();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P.n) {
        int64_t xi[3];
        load_particle<D, false>(pos, nullptr, i, xi);
        uint32_t c[3];
        cell_coords(P, keys[i], c);
        for_cells<D>(P, c, [&](uint32_t cell) {
            for (uint32_t j = max(start[cell], i + 1); j < start[cell + 1]; j++) {
                int64_t xj[3], d[3];
                load_particle<D, false>(pos, nullptr, j, xj);
#pragma unroll
                for (int a = 0; a < D; a++) d[a] = min_image(xj[a] - xi[a], P.box[a], P.half[a]);
                const int k = rdf_bin<D>(d, bins, scale, scalef, lim2f, margin);
                if (k >= 0) atomicAdd(&h[k], 1u);
            }
        });
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < bins; b += blockDim.x)
        if (h[b]) atomicAdd(out + b, (unsigned long long)h[b]);
}

// The same counts over every unordered pair, for boxes narrower than three cells of side rmax on
// some axis (small systems only). Positions are wrapped first: between list builds they may lie
// up to the skin outside [0, L).
template <int D>
__global__ void k_rdf_all(Params P, const Rec<D>* pos, uint32_t bins, double scale, float scalef, float lim2f, float margin,
                          unsigned long long* out) {
    extern __shared__ uint32_t h[];
    for (uint32_t b = threadIdx.x; b < bins; b += blockDim.x) h[b] = 0;
    __syncthreads();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P.n) {
        int64_t xi[3];
        load_particle<D, false>(pos, nullptr, i, xi);
        for (int a = 0; a < D; a++) xi[a] = wrap(xi[a], P.box[a]);
        for (uint32_t j = i + 1; j < P.n; j++) {
            int64_t xj[3], d[3];
            load_particle<D, false>(pos, nullptr, j, xj);
#pragma unroll
            for (int a = 0; a < D; a++) d[a] = min_image(wrap(xj[a], P.box[a]) - xi[a], P.box[a], P.half[a]);
            const int k = rdf_bin<D>(d, bins, scale, scalef, lim2f, margin);
            if (k >= 0) atomicAdd(&h[k], 1u);
        }
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < bins; b += blockDim.x)
        if (h[b]) atomicAdd(out + b, (unsigned long long)h[b]);
}

// Particle counts in slabs along one axis: min(floor(x / L * bins), bins - 1) in f64.
// Positions are wrapped first (between list builds they may lie up to the skin outside [0, L)).
// The f32 estimate x_f32 * (bins / L)_f32 is within 3 2^-24 bins (+ 2^-24 bins / L) of the
// exact quotient: a particle farther than `margin` from a slab edge takes its floor, the rest
// the f64 definition. Each block counts into shared memory and adds its counts once.
__device__ __forceinline__ uint32_t profile_bin(int64_t x, double l, uint32_t bins, float sf, float margin) {
    // x in [0, L): integer part (< 2^24 sigma) and the fraction's top 24 bits, each exact in f32
    const float xf = __fadd_rn(__int2float_rn((int32_t)(x >> 32)), __fmul_rn(__uint2float_rn((uint32_t)x >> 8), 0x1p-24f));
    const float t = __fmul_rn(xf, sf), fl = floorf(t), fr = __fsub_rn(t, fl);
    if (fr > margin && fr < 1.0f - margin) {
        const uint32_t k = (uint32_t)fl;
        return k < bins - 1 ? k : bins - 1;
    }
    return cell_of(x, l, bins);
}

template <int D>
__global__ void k_profile(uint32_t n, const Rec<D>* pos, uint32_t axis, int64_t lfix, double l, uint32_t bins, float sf, float margin,
                          unsigned long long* out) {
    extern __shared__ uint32_t h[];
    for (uint32_t b = threadIdx.x; b < bins; b += blockDim.x) h[b] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const long long* p = reinterpret_cast<const long long*>(pos + i);
        atomicAdd(&h[profile_bin(wrap(p[axis], lfix), l, bins, sf, margin)], 1u);
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < bins; b += blockDim.x)
        if (h[b]) atomicAdd(out + b, (unsigned long long)h[b]);
}

// The same with one global atomic per particle, for more bins than fit in shared memory.
template <int D>
__global__ void k_profile_wide(uint32_t n, const Rec<D>* pos, uint32_t axis, int64_t lfix, double l, uint32_t bins, unsigned long long* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long* p = reinterpret_cast<const long long*>(pos + i);
    atomicAdd(out + cell_of(wrap(p[axis], lfix), l, bins), 1ull);
}

// Observer::histogram (observe.wgsl:31-45): per particle the bin
// (min(u32(coord(x) sx), gx - 1), min(u32(coord(y) sy), gy - 1)), coord(x) = f32(x_hi) +
// f32(x_lo) 2^-32 in f32, of the wrapped position; counts of all particles in h[0, gx gy) and of
// the marked species in h[gx gy, 2 gx gy). Shared-memory counts when they fit (shm > 0), else one
// global atomic per count.
__device__ __forceinline__ uint32_t grid_bin(int64_t x, float scale, uint32_t g) {
    const float c = __fadd_rn(__uint2float_rn((uint32_t)((uint64_t)x >> 32)), __fmul_rn(__uint2float_rn((uint32_t)x), 0x1p-32f));
    const uint32_t b = __float2uint_rz(__fmul_rn(c, scale));
    return b < g - 1 ? b : g - 1;
}

__global__ void k_grid_hist(uint32_t n, const Rec<2>* pos, const uint32_t* species, int64_t lx, int64_t ly, float sx, float sy,
                            uint32_t gx, uint32_t gy, uint32_t marked, bool shm, uint32_t* out) {
    extern __shared__ uint32_t h[];
    const uint32_t bins = gx * gy;
    uint32_t* dst = shm ? h : out;
    if (shm) {
        for (uint32_t b = threadIdx.x; b < 2 * bins; b += blockDim.x) h[b] = 0;
        __syncthreads();
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const long long* p = reinterpret_cast<const long long*>(pos + i);
        const uint32_t b = grid_bin(wrap(p[1], ly), sy, gy) * gx + grid_bin(wrap(p[0], lx), sx, gx);
        atomicAdd(dst + b, 1u);
        if (species[i] == marked) atomicAdd(dst + bins + b, 1u);
    }
    if (shm) {
        __syncthreads();
        for (uint32_t b = threadIdx.x; b < 2 * bins; b += blockDim.x)
            if (h[b]) atomicAdd(out + b, h[b]);
    }
}

} // namespace

// Host memory that the device copies a frame into without the host waiting (pinned, grown on
// demand and kept for the engine's life).
static int pinned_grow(void** p, size_t* cap, size_t bytes) {
    if (bytes <= *cap) return GBMD_OK;
    pinned_give(*p, *cap);
    *cap = pin_class(bytes);
    *p = pinned_take(*cap);
    if (!*p) {
        *cap = 0;
        return fail(GBMD_E_NOMEM, "pinned frame buffer");
    }
    return GBMD_OK;
}

extern "C" int gbmd_observe_begin(gbmd_engine* e, uint32_t rdf_bins, double rdf_rmax, uint32_t profile_bins, uint32_t profile_axis) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    if (e->obs_pending) return fail(GBMD_E_INVALID, "a frame is already in flight (gbmd_observe_end first)");
    if (rdf_bins && (rdf_bins > 8192 || !(rdf_rmax > 0.0))) return fail(GBMD_E_INVALID, "bad RDF arguments");
    if (profile_bins && profile_axis >= (uint32_t)e->D) return fail(GBMD_E_INVALID, "bad profile arguments");
    GBMD_TRY(prepare_pairs_cond(e));
    GBMD_TRY(kicks_dispatch(e, nullptr, e->partial, 0));
    uint32_t n = e->n, nb = blocks_for(n, 128);
    GBMD_TRY(pinned_grow((void**)&e->obs_part_h, &e->obs_part_cap, 4 * (size_t)nb * 8));
    GBMD_CUDA_TRY(cudaMemcpyAsync(e->obs_part_h, e->partial, 4 * (size_t)nb * 8, cudaMemcpyDeviceToHost, e->st));
    size_t nbins = (size_t)rdf_bins + profile_bins;
    if (nbins > e->obs_bins_cap) {
        if (e->obs_bins) GBMD_CUDA_TRY(cudaFreeAsync(e->obs_bins, e->st));
        e->obs_bins = nullptr;
        e->obs_bins_cap = 0;
        if (cudaMallocAsync((void**)&e->obs_bins, nbins * 8, e->st) != cudaSuccess) return fail(GBMD_E_NOMEM, "observation bins");
        e->obs_bins_cap = nbins;
    }
    unsigned long long* dbuf = e->obs_bins;
    if (nbins) GBMD_CUDA_TRY(cudaMemsetAsync(dbuf, 0, nbins * 8, e->st));
    if (rdf_bins) {
        bool rdf_cells = true;
        double bmax = 0.0;
        for (int a = 0; a < e->D; a++) bmax = std::max(bmax, to_f64h(e->sys.box_len[a]));
        for (int a = 0; a < e->D; a++)
            if (std::floor(to_f64h(e->sys.box_len[a]) / (rdf_rmax + 1e-3 + 1e-6 * bmax)) < 3.0) rdf_cells = false;
        const double scale = (double)rdf_bins / rdf_rmax;
        const size_t shm = (size_t)rdf_bins * 4;
        // f32 fast path: beyond rmax (1 + 1e-4) for sure, or more than 1e-6 bins + 1e-5 from an edge
        const float scalef = (float)scale, lim2f = (float)(rdf_rmax * rdf_rmax * (1.0 + 1e-4));
        const float margin = (float)(1e-6 * rdf_bins + 1e-5);
        if (!rdf_cells) {
            if (e->D == 2)
                k_rdf_all<2><<<blocks_for(n, 128), 128, shm, e->st>>>(e->P, (const Rec<2>*)e->pos[e->cur], rdf_bins, scale, scalef, lim2f, margin, dbuf);
            else
                k_rdf_all<3><<<blocks_for(n, 128), 128, shm, e->st>>>(e->P, (const Rec<3>*)e->pos[e->cur], rdf_bins, scale, scalef, lim2f, margin, dbuf);
            note_launch();
        } else {
            // its own cell grid (side >= rmax) over the scratch buffers; the engine's own state,
            // lists and cell starts are untouched, so no list rebuild follows
            Params P = e->P;
            uint32_t nc[3];
            GBMD_TRY(cells_for(e->sys, rdf_rmax, nc));
            set_cells(P, nc, (uint32_t)e->D);
            size_t need = (size_t)P.ncell + 1;
            if (need > e->obs_start_cap) {
                if (e->obs_start) cudaFreeAsync(e->obs_start, e->st);
                e->obs_start = nullptr;
                e->obs_start_cap = 0;
                if (cudaMallocAsync((void**)&e->obs_start, need * 4, e->st) != cudaSuccess) return fail(GBMD_E_NOMEM, "RDF cell starts");
                e->obs_start_cap = need;
            }
            uint32_t* saved = e->start;
            e->start = e->obs_start;
            double wmax = 0.0;
            for (int a = 0; a < e->D; a++) wmax = std::max(wmax, (double)P.cell_w[a] * 0x1p-32);
            // The f32 offsets (relf, and each cell's base) lie within [-M, M), M the power of two
            // at or above 2 cell sides + 1; each carries a truncation below 2^-24 and a rounding of
            // at most M 2^-25, and so does their sum: per axis |d_f32 - d| <= delta. The sum of
            // squares, the square root and the product with the f32 scale add (D + 3) 2^-24
            // relatively. Twice the resulting bound, in bins, is the margin.
            double M = 1.0;
            while (M < 2.0 * wmax + 1.0) M *= 2.0;
            const bool narrow = M <= 64.0; // offsets >> 8 fit an int32
            const double delta = 2.0 * 0x1p-24 + 3.0 * M * 0x1p-25;
            const double err = std::sqrt((double)e->D) * delta + (rdf_rmax + 1.0) * (e->D + 3) * 0x1p-24;
            const float margin_c = (float)(2.0 * scale * err + 1e-5);
            const float lim2f_c = (float)((rdf_rmax + 2.0 * err) * (rdf_rmax + 2.0 * err) * (1.0 + 0x1p-20));
            if (e->D == 2) {
                enqueue_bin<2>(e, e->st, P);
                if (narrow)
                    k_rdf<2><<<blocks_for(n, 128), 128, shm, e->st>>>(P, (const Rec<2>*)e->pos_scr, e->relf, e->keys[e->sorted], e->start, rdf_bins,
                                                                     scale, scalef, lim2f_c, margin_c, dbuf);
                else
                    k_rdf_wide<2><<<blocks_for(n, 128), 128, shm, e->st>>>(P, (const Rec<2>*)e->pos_scr, e->keys[e->sorted], e->start, rdf_bins,
                                                                          scale, scalef, lim2f, margin, dbuf);
            } else {
                enqueue_bin<3>(e, e->st, P);
                if (narrow)
                    k_rdf<3><<<blocks_for(n, 128), 128, shm, e->st>>>(P, (const Rec<3>*)e->pos_scr, e->relf, e->keys[e->sorted], e->start, rdf_bins,
                                                                     scale, scalef, lim2f_c, margin_c, dbuf);
                else
                    k_rdf_wide<3><<<blocks_for(n, 128), 128, shm, e->st>>>(P, (const Rec<3>*)e->pos_scr, e->keys[e->sorted], e->start, rdf_bins,
                                                                          scale, scalef, lim2f, margin, dbuf);
            }
            note_launch();
            e->start = saved;
        }
    }
    if (profile_bins) {
        unsigned long long* pbuf = dbuf + rdf_bins;
        double l = to_f64h(e->sys.box_len[profile_axis]);
        int64_t lfix = e->P.box[profile_axis];
        if (profile_bins <= 8192 && l < 0x1p23) {
            const float sf = (float)((double)profile_bins / l);
            const float margin = (float)(4.0 * 0x1p-24 * profile_bins * (1.0 + 1.0 / l) + 1e-6);
            const uint32_t grid = std::min(blocks_for(n, 256), 1024u);
            const size_t shm = (size_t)profile_bins * 4;
            if (e->D == 2)
                k_profile<2><<<grid, 256, shm, e->st>>>(n, (const Rec<2>*)e->pos[e->cur], profile_axis, lfix, l, profile_bins, sf, margin, pbuf);
            else
                k_profile<3><<<grid, 256, shm, e->st>>>(n, (const Rec<3>*)e->pos[e->cur], profile_axis, lfix, l, profile_bins, sf, margin, pbuf);
        } else if (e->D == 2) {
            k_profile_wide<2><<<blocks_for(n, 256), 256, 0, e->st>>>(n, (const Rec<2>*)e->pos[e->cur], profile_axis, lfix, l, profile_bins, pbuf);
        } else {
            k_profile_wide<3><<<blocks_for(n, 256), 256, 0, e->st>>>(n, (const Rec<3>*)e->pos[e->cur], profile_axis, lfix, l, profile_bins, pbuf);
        }
        note_launch();
    }
    if (nbins) {
        GBMD_TRY(pinned_grow((void**)&e->obs_bins_h, &e->obs_bins_h_cap, nbins * 8));
        GBMD_CUDA_TRY(cudaMemcpyAsync(e->obs_bins_h, dbuf, nbins * 8, cudaMemcpyDeviceToHost, e->st));
    }
    GBMD_CUDA_TRY(cudaGetLastError());
    e->obs_pending = true;
    e->obs_rdf_bins = rdf_bins;
    e->obs_profile_bins = profile_bins;
    e->obs_nb = nb;
    return GBMD_OK;
}

extern "C" int gbmd_observe_grid(gbmd_engine* e, uint32_t gx, uint32_t gy, uint32_t marked, uint32_t* all, uint32_t* marked_counts,
                                 double* kinetic) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    if (e->D != 2) return fail(GBMD_E_UNSUPPORTED, "the density grid is two-dimensional (Observer takes a 2D engine)");
    if (e->obs_pending) return fail(GBMD_E_INVALID, "a frame is in flight (gbmd_observe_end first)");
    if (gx == 0 || gy == 0 || (uint64_t)gx * gy > (1u << 24)) return fail(GBMD_E_INVALID, "grid must have 1 to 2^24 bins");
    const uint32_t n = e->n, bins = gx * gy;
    uint32_t* d = nullptr;
    if (cudaMallocAsync((void**)&d, 2 * (size_t)bins * 4, e->st) != cudaSuccess) return fail(GBMD_E_NOMEM, "grid counts");
    std::vector<uint32_t> h(2 * (size_t)bins);
    std::vector<unsigned long long> part(8 * (size_t)e->thermo_nb);
    cudaError_t err = cudaMemsetAsync(d, 0, 2 * (size_t)bins * 4, e->st);
    if (err == cudaSuccess) {
        // scale = (g / L) as f32 (observe.rs:58): the f64 quotient rounded once
        const float sx = (float)((double)gx / to_f64h(e->sys.box_len[0])), sy = (float)((double)gy / to_f64h(e->sys.box_len[1]));
        const bool shm = 2 * (size_t)bins * 4 <= 48 * 1024;
        const uint32_t grid = shm ? std::min(blocks_for(n, 256), 1024u) : blocks_for(n, 256);
        k_grid_hist<<<std::max(grid, 1u), 256, shm ? 2 * (size_t)bins * 4 : 0, e->st>>>(n, (const Rec<2>*)e->pos[e->cur], e->species, e->P.box[0],
                                                                                           e->P.box[1], sx, sy, gx, gy, marked, shm, d);
        k_ke_exact<2><<<e->thermo_nb, 256, 0, e->st>>>(n, e->vel, e->species, e->sys.pinned, e->tpart);
        note_launch(2);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = cudaMemcpyAsync(h.data(), d, 2 * (size_t)bins * 4, cudaMemcpyDeviceToHost, e->st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(part.data(), e->tpart, part.size() * 8, cudaMemcpyDeviceToHost, e->st);
    cudaFreeAsync(d, e->st);
    GBMD_CUDA_TRY(err);
    GBMD_CUDA_TRY(cudaStreamSynchronize(e->st));
    if (all) std::memcpy(all, h.data(), (size_t)bins * 4);
    if (marked_counts) std::memcpy(marked_counts, h.data() + bins, (size_t)bins * 4);
    if (kinetic) {
        // sum_s 1/2 m_s S_s (UNIT / dt)^2, S_s the exact sum of v^2 over the moving particles of s
        const double u = (1.0 / 4294967296.0) / e->sys.dt;
        double ke = 0.0;
        for (uint32_t s = 0; s < e->sys.nspecies; s++) {
            unsigned __int128 S = 0;
            for (uint32_t b = 0; b < e->thermo_nb; b++) S += ((unsigned __int128)part[8 * b + 2 * s + 1] << 64) | part[8 * b + 2 * s];
            const double sum = (double)(uint64_t)(S >> 64) * 18446744073709551616.0 + (double)(uint64_t)S;
            ke += 0.5 * e->sys.masses[s] * sum * (u * u);
        }
        *kinetic = ke;
    }
    return GBMD_OK;
}

extern "C" int gbmd_observe_end(gbmd_engine* e, gbmd_frame* frame, uint64_t* rdf, uint64_t* profile) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    if (!e->obs_pending) return fail(GBMD_E_INVALID, "no frame in flight (gbmd_observe_begin first)");
    e->obs_pending = false;
    GBMD_CUDA_TRY(cudaStreamSynchronize(e->st)); // returns at once when the frame's work is done
    GBMD_TRY(check_ctl(e));
    if (rdf && e->obs_rdf_bins) std::memcpy(rdf, e->obs_bins_h, (size_t)e->obs_rdf_bins * 8);
    if (profile && e->obs_profile_bins) std::memcpy(profile, e->obs_bins_h + e->obs_rdf_bins, (size_t)e->obs_profile_bins * 8);
    if (frame) {
        const uint32_t n = e->n, nb = e->obs_nb;
        const double* part = e->obs_part_h;
        double pe = 0.0, w = 0.0, ke = 0.0, gpe = 0.0;
        for (uint32_t b = 0; b < nb; b++) {
            pe += part[4 * b];
            w += part[4 * b + 1];
            ke += part[4 * b + 2];
            gpe += part[4 * b + 3];
        }
        ke *= 0x1p-64 / (8.0 * e->sys.dt * e->sys.dt); // sum of m (v + next)^2 -> 0.5 m vh^2 (k_kicks)
        pe += gpe;
        double vol = 1.0;
        for (int a = 0; a < e->D; a++) vol *= to_f64h(e->sys.box_len[a]);
        double dof = 0.5 * e->D * std::max((double)n - 1.0, 1.0);
        frame->step = (uint64_t)e->steps;
        frame->kinetic = ke;
        frame->potential = pe;
        frame->virial = w;
        frame->temperature = ke / dof;
        frame->pressure = (double)n / vol * frame->temperature + w / (e->D * vol);
        frame->volume = vol;
        frame->n = n;
        frame->dim = (uint32_t)e->D;
        if (!std::isfinite(ke) || !std::isfinite(pe) || !std::isfinite(w))
            return fail(GBMD_E_NONFINITE, "a non-finite energy or virial (the frame is filled in)");
    }
    return GBMD_OK;
}

// ------------------------------------------------------------------ checkpoint / resume
// Snapshot layout (little-endian): 8-byte magic "GBMDSNP1"; u32 version (1), dim, n, reserved;
// i64 steps; u32 clock, reserved; u64 thermostat phase; u64 State::hash of the arrays; then the
// id-ordered positions (i64 x dim x n), velocities (i32 x dim x n) and species (u32 x n).
namespace {
constexpr char SNAP_MAGIC[8] = {'G', 'B', 'M', 'D', 'S', 'N', 'P', '1'};
constexpr size_t SNAP_HEADER = 8 + 4 * 4 + 8 + 4 * 2 + 8 + 8;
} // namespace

extern "C" size_t gbmd_snapshot_bytes(uint32_t dim, uint32_t n) { return SNAP_HEADER + (size_t)n * (dim * 8 + dim * 4 + 4); }

extern "C" int gbmd_snapshot(gbmd_engine* e, void* buf, size_t cap, size_t* written) {
    if (!e || !buf) return fail(GBMD_E_INVALID, "null argument");
    const size_t need = gbmd_snapshot_bytes((uint32_t)e->D, e->n), D = (size_t)e->D, n = e->n;
    if (cap < need) return fail(GBMD_E_INVALID, "snapshot buffer too small (gbmd_snapshot_bytes)");
    char* p = (char*)buf;
    int64_t* pos = (int64_t*)(p + SNAP_HEADER);
    int32_t* vel = (int32_t*)(p + SNAP_HEADER + n * D * 8);
    uint32_t* sp = (uint32_t*)(p + SNAP_HEADER + n * D * 12);
    GBMD_TRY(gbmd_read_state(e, pos, vel, sp));
    const uint64_t h = gbmd_hash_state((uint32_t)D, pos, vel, sp, e->n);
    const uint32_t head[4] = {1u, (uint32_t)D, e->n, 0u}, clk[2] = {e->clock, 0u};
    const int64_t steps = e->steps;
    const uint64_t tc = e->tcount;
    std::memcpy(p, SNAP_MAGIC, 8);
    std::memcpy(p + 8, head, 16);
    std::memcpy(p + 24, &steps, 8);
    std::memcpy(p + 32, clk, 8);
    std::memcpy(p + 40, &tc, 8);
    std::memcpy(p + 48, &h, 8);
    if (written) *written = need;
    return GBMD_OK;
}

extern "C" int gbmd_restore(gbmd_engine* e, const void* buf, size_t size) {
    if (!e || !buf) return fail(GBMD_E_INVALID, "null argument");
    const char* p = (const char*)buf;
    if (size < SNAP_HEADER || std::memcmp(p, SNAP_MAGIC, 8) != 0) return fail(GBMD_E_INVALID, "not a snapshot (magic)");
    uint32_t head[4], clk[2];
    int64_t steps;
    uint64_t tc, h;
    std::memcpy(head, p + 8, 16);
    std::memcpy(&steps, p + 24, 8);
    std::memcpy(clk, p + 32, 8);
    std::memcpy(&tc, p + 40, 8);
    std::memcpy(&h, p + 48, 8);
    if (head[0] != 1u) return fail(GBMD_E_INVALID, "unknown snapshot version");
    if (head[1] != (uint32_t)e->D || head[2] != e->n) return fail(GBMD_E_INVALID, "snapshot of another dimension or particle count");
    if (size != gbmd_snapshot_bytes(head[1], head[2])) return fail(GBMD_E_INVALID, "snapshot size does not match its header");
    const size_t D = head[1], n = head[2];
    const int64_t* pos = (const int64_t*)(p + SNAP_HEADER);
    const int32_t* vel = (const int32_t*)(p + SNAP_HEADER + n * D * 8);
    const uint32_t* sp = (const uint32_t*)(p + SNAP_HEADER + n * D * 12);
    if (gbmd_hash_state((uint32_t)D, pos, vel, sp, (uint32_t)n) != h) return fail(GBMD_E_INVALID, "snapshot corrupted (state hash mismatch)");
    GBMD_TRY(gbmd_upload(e, pos, vel, sp));
    e->steps = steps;
    e->clock = clk[0];
    e->tcount = tc;
    return gbmd_sync(e);
}

extern "C" int gbmd_observe(gbmd_engine* e, gbmd_frame* frame, uint64_t* rdf, uint32_t rdf_bins, double rdf_rmax, uint64_t* profile,
                            uint32_t profile_bins, uint32_t profile_axis) {
    if (!e) return fail(GBMD_E_INVALID, "null engine");
    if (rdf && (rdf_bins == 0 || rdf_bins > 8192 || !(rdf_rmax > 0.0))) return fail(GBMD_E_INVALID, "bad RDF arguments");
    if (profile && (profile_bins == 0 || profile_axis >= (uint32_t)e->D)) return fail(GBMD_E_INVALID, "bad profile arguments");
    GBMD_TRY(gbmd_observe_begin(e, rdf ? rdf_bins : 0, rdf_rmax, profile ? profile_bins : 0, profile_axis));
    return gbmd_observe_end(e, frame, rdf, profile);
}

// ------------------------------------------------------------------ seeded init + hashing
namespace {
__global__ void k_libm(uint32_t n, const double* x, double* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[3 * (size_t)i] = dev_log(x[i]);
    out[3 * (size_t)i + 1] = dev_cos(x[i]);
    out[3 * (size_t)i + 2] = dev_sin(x[i]);
}
} // namespace

// The device's ln, cos and sin (the fdlibm restatement the initial velocities, the heat bath and
// thermal walls draw with) at n arguments: out[3 i .. 3 i + 2].
extern "C" int gbmd_debug_libm(const double* x, uint32_t n, double* out) {
    if ((n && (!x || !out))) return fail(GBMD_E_INVALID, "null argument");
    if (n == 0) return GBMD_OK;
    cudaStream_t s;
    GBMD_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    double *dx = nullptr, *dout = nullptr;
    int rc = GBMD_OK;
    if (cudaMallocAsync((void**)&dx, (size_t)n * 8, s) != cudaSuccess || cudaMallocAsync((void**)&dout, (size_t)n * 24, s) != cudaSuccess)
        rc = fail(GBMD_E_NOMEM, "libm buffers");
    if (rc == GBMD_OK) {
        cudaMemcpyAsync(dx, x, (size_t)n * 8, cudaMemcpyHostToDevice, s);
        k_libm<<<blocks_for(n, 256), 256, 0, s>>>(n, dx, dout);
        note_launch();
        cudaMemcpyAsync(out, dout, (size_t)n * 24, cudaMemcpyDeviceToHost, s);
        const cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = fail(GBMD_E_CUDA, cudaGetErrorString(e));
    }
    if (dx) cudaFreeAsync(dx, s);
    if (dout) cudaFreeAsync(dout, s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return rc;
}

extern "C" int gbmd_init_state(const gbmd_system* sys, const gbmd_init* spec, int64_t* pos, int32_t* vel, uint32_t* species) {
    if (!sys || !spec) return fail(GBMD_E_INVALID, "null argument");
    GBMD_TRY(validate_system(*sys, spec->n));
    size_t n = spec->n, D = sys->dim;
    if (n == 0) return GBMD_OK;
    cudaStream_t s;
    GBMD_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    void* dpos = nullptr;
    int32_t* dvel = nullptr;
    uint32_t* dsp = nullptr;
    int rc = GBMD_OK;
    // (stream-ordered: a server creates states while other requests run)
    if (cudaMallocAsync(&dpos, n * (D == 2 ? 16 : 32), s) != cudaSuccess || cudaMallocAsync((void**)&dvel, n * D * 4, s) != cudaSuccess ||
        cudaMallocAsync((void**)&dsp, n * 4, s) != cudaSuccess)
        rc = fail(GBMD_E_NOMEM, "init buffers");
    if (rc == GBMD_OK) rc = init_state_device(*sys, *spec, dpos, dvel, dsp, s);
    std::vector<int64_t> rec;
    if (rc == GBMD_OK) {
        rec.resize(n * (D == 2 ? 2 : 4));
        if (cudaMemcpyAsync(rec.data(), dpos, rec.size() * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess) rc = fail(GBMD_E_CUDA, "copy");
        if (vel && cudaMemcpyAsync(vel, dvel, n * D * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) rc = fail(GBMD_E_CUDA, "copy");
        if (species && cudaMemcpyAsync(species, dsp, n * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) rc = fail(GBMD_E_CUDA, "copy");
        cudaError_t err = cudaStreamSynchronize(s);
        if (err != cudaSuccess) rc = fail(GBMD_E_CUDA, cudaGetErrorString(err));
    }
    if (rc == GBMD_OK && pos) {
        size_t w = D == 2 ? 2 : 4;
        for (size_t i = 0; i < n; i++)
            for (size_t a = 0; a < D; a++) pos[D * i + a] = rec[w * i + a];
    }
    if (dpos) cudaFreeAsync(dpos, s);
    if (dvel) cudaFreeAsync(dvel, s);
    if (dsp) cudaFreeAsync(dsp, s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return rc;
}

static int velocities_on_device(const gbmd_system* sys, const uint32_t* species, uint32_t n, double t, uint64_t seed, int32_t* vel,
                                bool fixed_speed) {
    if (!sys || (n && (!species || !vel))) return fail(GBMD_E_INVALID, "null argument");
    GBMD_TRY(validate_system(*sys, n));
    for (uint32_t i = 0; i < n; i++)
        if (species[i] >= sys->nspecies) return fail(GBMD_E_INVALID, "species out of range");
    if (n == 0) return GBMD_OK;
    const size_t D = sys->dim;
    cudaStream_t s;
    GBMD_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    int32_t* dvel = nullptr;
    uint32_t* dsp = nullptr;
    int rc = GBMD_OK;
    if (cudaMallocAsync((void**)&dvel, n * D * 4, s) != cudaSuccess || cudaMallocAsync((void**)&dsp, (size_t)n * 4, s) != cudaSuccess)
        rc = fail(GBMD_E_NOMEM, "maxwell buffers");
    if (rc == GBMD_OK && cudaMemcpyAsync(dsp, species, (size_t)n * 4, cudaMemcpyHostToDevice, s) != cudaSuccess) rc = fail(GBMD_E_CUDA, "copy");
    if (rc == GBMD_OK) rc = maxwell_state_device(*sys, n, t, seed, dsp, dvel, s, fixed_speed);
    if (rc == GBMD_OK && cudaMemcpyAsync(vel, dvel, n * D * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) rc = fail(GBMD_E_CUDA, "copy");
    if (rc == GBMD_OK) {
        cudaError_t err = cudaStreamSynchronize(s);
        if (err != cudaSuccess) rc = fail(GBMD_E_CUDA, cudaGetErrorString(err));
    }
    if (dvel) cudaFreeAsync(dvel, s);
    if (dsp) cudaFreeAsync(dsp, s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return rc;
}

extern "C" int gbmd_maxwell(const gbmd_system* sys, const uint32_t* species, uint32_t n, double t, uint64_t seed, int32_t* vel) {
    return velocities_on_device(sys, species, n, t, seed, vel, false);
}
extern "C" int gbmd_fixed_speed(const gbmd_system* sys, const uint32_t* species, uint32_t n, double t, uint64_t seed, int32_t* vel) {
    if (sys && sys->dim != 2) return fail(GBMD_E_UNSUPPORTED, "fixed_speed is two-dimensional (init::fixed_speed)");
    return velocities_on_device(sys, species, n, t, seed, vel, true);
}

// FNV-1a of an id-ordered state (State::hash, system.rs:460-477; State3::hash, three.rs:281-297).
extern "C" uint64_t gbmd_hash_state(uint32_t dim, const int64_t* pos, const int32_t* vel, const uint32_t* species, uint32_t n) {
    uint64_t h = 0xcbf29ce484222325ull;
    auto eat = [&](const void* p, size_t len) {
        const uint8_t* b = (const uint8_t*)p;
        for (size_t k = 0; k < len; k++) {
            h ^= b[k];
            h *= 0x100000001b3ull;
        }
    };
    for (size_t i = 0; i < n; i++) {
        if (dim == 2) {
            eat(&pos[2 * i], 8);
            eat(&pos[2 * i + 1], 8);
            eat(&vel[2 * i], 4);
            eat(&vel[2 * i + 1], 4);
        } else {
            for (int a = 0; a < 3; a++) {
                eat(&pos[3 * i + a], 8);
                eat(&vel[3 * i + a], 4);
            }
        }
        eat(&species[i], 4);
    }
    return h;
}
