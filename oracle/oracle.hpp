// ORACLE — test infrastructure only. Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline may load it, as the checker; the engine never links or calls it.
//
// A C++17 restatement of micrographia's CPU semantics for the integer fixed-point LJ path:
//   gpu-prims: threefry.rs (Threefry-2x32, uniforms, Box–Muller), fixed64.rs
//   md-core:   fixed.rs, pair.rs, system.rs (System/State subset), init.rs, three.rs, table.rs
//   md-ref:    real.rs (f32/f64 Real semantics), cells.rs, int_engine.rs and int_engine3.rs
//              (periodic or walled boxes, the Andersen bath, the ledger), fast.rs (the SIMD fast
//              path: the timed CPU baseline),
//              float_engine.rs
//   md:        the Verlet-list definition of shaders/neighbors.wgsl:27-64 / md3.wgsl:443-483
// plus f64 instruments the reference lacks (virial pressure after mc/src/gibbs.rs:58-66,
// 381-390; RDF; density profile; exact-integer velocity rescale).
//
// Rust semantics restated exactly: `as` float->int casts saturate and send NaN to 0; i32 sums
// wrap; `round_ties_even` is rint in the default rounding mode; `f64::round` is round();
// nothing is contracted into FMAs (compile with -ffp-contract=off, no fast-math).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "../include/gbmd.h"
#include "fdlibm.hpp"

namespace oracle {

// ---------------------------------------------------------------- Rust cast semantics
inline int32_t sat_i32(double x) {
    if (x != x) return 0;
    if (x >= 2147483647.0) return INT32_MAX;
    if (x <= -2147483648.0) return INT32_MIN;
    return (int32_t)x;
}
inline int32_t sat_i32f(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x <= -2147483648.0f) return INT32_MIN;
    return (int32_t)x;
}
inline uint32_t sat_u32(double x) {
    if (!(x > 0.0)) return 0;
    if (x >= 4294967295.0) return UINT32_MAX;
    return (uint32_t)x;
}
inline int64_t sat_i64(double x) {
    if (x != x) return 0;
    if (x >= 9223372036854775807.0) return INT64_MAX;
    if (x <= -9223372036854775808.0) return INT64_MIN;
    return (int64_t)x;
}
inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
inline int32_t wneg(int32_t a) { return (int32_t)(0u - (uint32_t)a); }
inline int64_t div_euclid(int64_t a, int64_t b) {
    int64_t q = a / b, r = a % b;
    if (r < 0) q = b > 0 ? q - 1 : q + 1;
    return q;
}
inline int64_t rem_euclid(int64_t a, int64_t b) {
    int64_t r = a % b;
    if (r < 0) r += b < 0 ? -b : b;
    return r;
}
// LLVM's expansion of powi(x, n) for a constant n > 0 (binary powering, as compiler-rt's
// __powidf2): the result Rust's f64::powi gives.
inline double powi(double x, int n) {
    double res = 1.0;
    bool have = false;
    double sq = x;
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

// ---------------------------------------------------------------- gpu-prims/src/threefry.rs
inline uint32_t rotl(uint32_t x, uint32_t r) { return (x << r) | (x >> (32 - r)); }
// threefry.rs:7-22
inline std::array<uint32_t, 2> threefry2x32_rounds(std::array<uint32_t, 2> ctr, std::array<uint32_t, 2> key, uint32_t rounds) {
    static const uint32_t ROT[8] = {13, 15, 26, 6, 17, 29, 16, 24};
    const uint32_t ks[3] = {key[0], key[1], 0x1BD11BDAu ^ key[0] ^ key[1]};
    uint32_t x0 = ctr[0] + ks[0];
    uint32_t x1 = ctr[1] + ks[1];
    for (uint32_t r = 0; r < rounds; r++) {
        x0 += x1;
        x1 = rotl(x1, ROT[r % 8]);
        x1 ^= x0;
        if ((r & 3) == 3) {
            uint32_t s = (r >> 2) + 1;
            x0 += ks[s % 3];
            x1 += ks[(s + 1) % 3] + s;
        }
    }
    return {x0, x1};
}
inline std::array<uint32_t, 2> threefry2x32(std::array<uint32_t, 2> ctr, std::array<uint32_t, 2> key) {
    return threefry2x32_rounds(ctr, key, 20);
}
// threefry.rs:29-32
inline double to_unit_f64(std::array<uint32_t, 2> r) {
    uint64_t b = ((uint64_t)r[0] << 21) ^ ((uint64_t)r[1] >> 11);
    return (double)(b & ((1ull << 53) - 1)) * (1.0 / 9007199254740992.0);
}
// threefry.rs:35-37
inline double uniform(uint64_t seed, uint32_t stream, uint32_t i) {
    return to_unit_f64(threefry2x32({i, stream}, {(uint32_t)seed, (uint32_t)(seed >> 32)}));
}
// threefry.rs:42-46 (libm sqrt, log, cos)
inline double normal(uint64_t seed, uint32_t stream, uint32_t i) {
    double u1 = 1.0 - uniform(seed, stream, 2 * i);
    double u2 = uniform(seed, stream, 2 * i + 1);
    return std::sqrt(-2.0 * fdlibm::log(u1)) * fdlibm::cos(6.28318530717958647692 * u2);
}

// ---------------------------------------------------------------- md-core/src/fixed.rs
constexpr int64_t ONE = (int64_t)1 << 32;
constexpr double UNIT = 1.0 / 4294967296.0;
constexpr int64_t SEP_LIMIT = 8 * ONE;
constexpr float SEP_UNIT_F32 = 1.0f / 268435456.0f; /* 2^-28 */

inline int64_t to_fixed(double x) { return sat_i64(std::round(x * 4294967296.0)); } // fixed.rs:21-23
inline double to_f64(int64_t x) { return (double)x * UNIT; }                       // fixed.rs:25-27
inline int64_t min_image(int64_t a, int64_t b, int64_t l) {                         // fixed.rs:31-40
    int64_t d = b - a, half = l / 2;
    if (d >= half) d -= l;
    else if (d < -half) d += l;
    return d;
}
inline int64_t wrap(int64_t x, int64_t l) { return x < 0 ? x + l : (x >= l ? x - l : x); } // 43-51
// fixed.rs:55-61: separation as f32 through 2^-28 sigma units, or none beyond 8 sigma.
inline bool sep_f32(int64_t d, float* out) {
    if (!(d >= -SEP_LIMIT && d < SEP_LIMIT)) return false;
    uint64_t m = d < 0 ? (uint64_t)0 - (uint64_t)d : (uint64_t)d;
    float mag = (float)(uint32_t)(m >> 4) * SEP_UNIT_F32;
    *out = d < 0 ? -mag : mag;
    return true;
}
// fixed.rs:63-72: sep_f32 within 8 sigma; beyond, the magnitude's whole sigma plus its fraction
// in f32, then the sign (bonds can be longer than the pair separation handles).
inline float sep_long_f32(int64_t d) {
    float s;
    if (sep_f32(d, &s)) return s;
    const uint64_t m = d < 0 ? (uint64_t)0 - (uint64_t)d : (uint64_t)d;
    const float mag = (float)(uint32_t)(m >> 32) + (float)(uint32_t)m * (1.0f / 4294967296.0f);
    return d < 0 ? -mag : mag;
}
// md-ref real.rs:59-64: branch-free sep for |d| < 8 sigma, bit-identical to sep_f32.
inline float sep_near_f32(int64_t d) {
    int64_t q = (d + ((d >> 63) & 15)) >> 4;
    float v = (float)(int32_t)q * SEP_UNIT_F32;
    uint32_t vb;
    std::memcpy(&vb, &v, 4);
    vb |= (uint32_t)(d >> 32) & 0x80000000u;
    std::memcpy(&v, &vb, 4);
    return v;
}

// ---------------------------------------------------------------- md-core/src/pair.rs
struct Pair {
    double eps = 1.0, sigma = 1.0, rc = 2.5;
    static Pair lj(double rc) { return {1.0, 1.0, rc}; }
    static Pair wca() { return {1.0, 1.0, std::pow(2.0, 1.0 / 6.0)}; }
    double shift() const { // pair.rs:28-34
        if (eps == 0.0 || rc == 0.0) return 0.0;
        double s6 = powi(sigma / rc, 6);
        return 4.0 * eps * s6 * (s6 - 1.0);
    }
    double energy(double r2) const { // pair.rs:36-42
        if (r2 >= rc * rc) return 0.0;
        double s6 = powi(sigma * sigma / r2, 3);
        return 4.0 * eps * s6 * (s6 - 1.0) - shift();
    }
    double f_over_r(double r2) const { // pair.rs:45-51
        if (r2 >= rc * rc) return 0.0;
        double s6 = powi(sigma * sigma / r2, 3);
        return 24.0 * eps * s6 * (2.0 * s6 - 1.0) / r2;
    }
};

// ---------------------------------------------------------------- md-core System / System3
// The Andersen heat bath: md_core::Thermostat (system.rs:156-175) in 2D, three::Bath
// (three.rs:79-83) in 3D, which has only t, rate and species.
struct Bath {
    bool on = false;
    double t = 0.0, rate = 0.0, drift = 0.0;
    uint32_t species = 0xffffffffu;
    int axis = 0;
    int64_t region[2] = {INT64_MIN, INT64_MAX};
};

// The periodic LJ subset of System (system.rs:26-64) and System3 (three.rs:13-31), with the bath.
struct System {
    int dim = 2;
    std::array<int64_t, 3> box{0, 0, 0};
    double dt = 0.005;
    std::vector<double> masses{1.0};
    std::vector<Pair> pairs{Pair::lj(2.5)};
    std::array<double, 3> gravity{0, 0, 0};
    uint64_t seed = 1;
    uint32_t pinned = 0;
    Bath bath;
    // Walls (md_core::Wall, walls.rs) on the axes whose periodic bit is clear: GBMD_WALL_* per side.
    uint32_t periodic_bits = 7;
    std::array<std::array<uint32_t, 2>, 3> wall_kind{};
    std::array<std::array<double, 2>, 3> wall_t{};
    bool periodic(int a) const { return (periodic_bits >> a) & 1u; } // system.rs:384-386
    // md_core::Membrane (system.rs:119-141), 2D
    bool membrane = false;
    int membrane_axis = 0;
    uint32_t membrane_blocks = 0, membrane_pore_shift = 0;
    int64_t membrane_position = 0, membrane_pore_width = 0;
    bool membrane_blocks_species(uint32_t s) const { return (membrane_blocks >> s) & 1u; }
    // compartments (system.rs:222-257), 2D: shift per axis (0: none), insulating or diathermal
    uint32_t compartments[2] = {0, 0};
    bool diathermal = false;
    int64_t compartment_of(const int64_t* p, int a) const { return compartments[a] == 0 ? 0 : p[a] >> compartments[a]; }
    bool interact_across(const int64_t* a, const int64_t* b) const { // system.rs:229-231
        return dim != 2 || diathermal || (compartment_of(a, 0) == compartment_of(b, 0) && compartment_of(a, 1) == compartment_of(b, 1));
    }
    bool in_pore(int64_t along) const {
        return membrane_pore_shift != 0 && (along & (((int64_t)1 << membrane_pore_shift) - 1)) < membrane_pore_width;
    }
    bool all_periodic() const { return (periodic_bits & ((1u << dim) - 1u)) == ((1u << dim) - 1u); }

    static System from_c(const gbmd_system& s) {
        System o;
        o.dim = (int)s.dim;
        for (int a = 0; a < 3; a++) o.box[a] = s.box_len[a];
        o.dt = s.dt;
        o.masses.assign(s.masses, s.masses + s.nspecies);
        o.pairs.clear();
        for (uint32_t k = 0; k < s.nspecies * s.nspecies; k++) o.pairs.push_back({s.pairs[k].eps, s.pairs[k].sigma, s.pairs[k].rc});
        for (int a = 0; a < 3; a++) o.gravity[a] = s.gravity[a];
        o.seed = s.seed;
        o.pinned = s.pinned;
        o.periodic_bits = s.periodic | (s.dim == 2 ? 4u : 0u);
        o.compartments[0] = s.dim == 2 ? s.compartments[0] : 0;
        o.compartments[1] = s.dim == 2 ? s.compartments[1] : 0;
        o.diathermal = s.compartments_diathermal != 0;
        o.membrane = s.membrane != 0;
        o.membrane_axis = (int)s.membrane_axis;
        o.membrane_blocks = s.membrane_blocks;
        o.membrane_pore_shift = s.membrane_pore_shift;
        o.membrane_position = s.membrane_position;
        o.membrane_pore_width = s.membrane_pore_width;
        for (int a = 0; a < 3; a++)
            for (int side = 0; side < 2; side++) {
                o.wall_kind[a][side] = s.wall_kind[a][side];
                o.wall_t[a][side] = s.wall_t[a][side];
            }
        if (s.bath) {
            o.bath.on = true;
            o.bath.t = s.bath_t;
            o.bath.rate = s.bath_rate;
            o.bath.drift = s.bath_drift;
            o.bath.species = s.bath_species;
            o.bath.axis = (int)s.bath_axis;
            o.bath.region[0] = s.bath_region[0];
            o.bath.region[1] = s.bath_region[1];
        }
        return o;
    }
    int species() const { return (int)masses.size(); }
    const Pair& pair(uint32_t a, uint32_t b) const { return pairs[a * masses.size() + b]; }
    bool is_pinned(uint32_t s) const { return (pinned >> s) & 1u; }
    double rc_max() const {
        double r = 0.0;
        for (auto& p : pairs) r = std::max(r, p.rc);
        return r;
    }
    double box_f64(int a) const { return to_f64(box[a]); }
    double volume() const {
        double v = 1.0;
        for (int a = 0; a < dim; a++) v *= box_f64(a);
        return v;
    }
    // system.rs:415-420 / three.rs:134-139
    double kick_coeff(uint32_t s) const {
        if (is_pinned(s)) return 0.0;
        return dt * dt / masses[s] * 4294967296.0;
    }
    double velocity(int32_t v) const { return (double)v * UNIT / dt; }                      // 423-425
    int32_t to_step_displacement(double v) const { return sat_i32(std::round(v * dt * 4294967296.0)); } // 427-429
    // system.rs:399-402: the same for every species.
    std::array<int32_t, 3> gravity_kick() const {
        std::array<int32_t, 3> g{0, 0, 0};
        for (int a = 0; a < dim; a++) g[a] = sat_i32(std::round(gravity[a] * dt * dt * 4294967296.0));
        return g;
    }
    // system.rs:438-444 / three.rs:151-157
    std::array<uint32_t, 3> cells_for(double r) const {
        double bmax = 0.0;
        for (int a = 0; a < dim; a++) bmax = std::max(bmax, box_f64(a));
        double margin = 1e-3 + 1e-6 * bmax;
        std::array<uint32_t, 3> c{1, 1, 1};
        for (int a = 0; a < dim; a++) {
            c[a] = sat_u32(std::floor(box_f64(a) / (r + margin)));
            if (c[a] < 3) throw std::invalid_argument("box too small for the cell radius");
        }
        return c;
    }
};

// Positions, half-step velocities and species, interleaved like md-core's State / State3.
struct State {
    int dim = 2;
    std::vector<int64_t> pos; // n * dim
    std::vector<int32_t> vel; // n * dim
    std::vector<uint32_t> species;
    size_t n() const { return species.size(); }
    // system.rs:460-477 (2D: x, y, vx, vy, s) and three.rs:281-297 (3D: (x, vx) per axis, s).
    uint64_t hash() const {
        uint64_t h = 0xcbf29ce484222325ull;
        auto eat = [&](const void* p, size_t len) {
            const uint8_t* b = (const uint8_t*)p;
            for (size_t k = 0; k < len; k++) {
                h ^= b[k];
                h *= 0x100000001b3ull;
            }
        };
        for (size_t i = 0; i < n(); i++) {
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
};

// ---------------------------------------------------------------- md-core/src/init.rs
constexpr uint32_t STREAM_VELOCITY = 1, STREAM_JITTER = 2, STREAM_DIRECTION = 3;
// New streams of this engine's own recipes (slab vapour placement).
constexpr uint32_t STREAM_VAPOUR = 4;

// init.rs:15-19
inline std::array<int64_t, 2> box_for(size_t n, double density, double aspect) {
    double area = (double)n / density;
    double ly = std::sqrt(area / aspect);
    return {to_fixed(ly * aspect), to_fixed(ly)};
}
// init.rs:22-38
inline std::vector<int64_t> lattice(size_t n, std::array<int64_t, 2> box, double jitter, uint64_t seed) {
    double b0 = to_f64(box[0]), b1 = to_f64(box[1]);
    size_t nx = std::max<size_t>((size_t)sat_u32(std::ceil(std::sqrt((double)n * b0 / b1))), 1);
    size_t ny = (n + nx - 1) / nx;
    double a0 = b0 / (double)nx, a1 = b1 / (double)ny;
    std::vector<int64_t> pos(2 * n);
    for (size_t k = 0; k < n; k++) {
        size_t i = k % nx, j = k / nx;
        double jx = jitter * (uniform(seed, STREAM_JITTER, 2 * (uint32_t)k) - 0.5);
        double jy = jitter * (uniform(seed, STREAM_JITTER, 2 * (uint32_t)k + 1) - 0.5);
        pos[2 * k] = wrap(to_fixed(((double)i + 0.5) * a0 + jx), box[0]);
        pos[2 * k + 1] = wrap(to_fixed(((double)j + 0.5) * a1 + jy), box[1]);
    }
    return pos;
}
// init.rs:76-89 (2D) and three.rs:376-389 (over moving particles; pinned excluded).
inline void zero_velocity_sum(const System& sys, const std::vector<uint32_t>& species, std::vector<int32_t>& vel, bool skip_pinned) {
    int d = sys.dim;
    size_t n = species.size();
    std::vector<size_t> moving;
    for (size_t i = 0; i < n; i++)
        if (!skip_pinned || !sys.is_pinned(species[i])) moving.push_back(i);
    int64_t m = (int64_t)moving.size();
    if (m == 0) return;
    for (int a = 0; a < d; a++) {
        int64_t sum = 0;
        for (size_t i : moving) sum += vel[d * i + a];
        int64_t q = div_euclid(sum, m), r = rem_euclid(sum, m);
        for (size_t k = 0; k < moving.size(); k++) {
            size_t i = moving[k];
            vel[d * i + a] = wadd(vel[d * i + a], wneg((int32_t)(q + ((int64_t)k < r ? 1 : 0))));
        }
    }
}
// init.rs:42-57 (2D; counter 2i + a) and three.rs:359-373 (3D; counter 3i + a, pinned -> 0).
inline std::vector<int32_t> maxwell(const System& sys, const std::vector<uint32_t>& species, double t, uint64_t seed) {
    int d = sys.dim;
    size_t n = species.size();
    std::vector<int32_t> vel(d * n, 0);
    for (size_t i = 0; i < n; i++) {
        uint32_t s = species[i];
        if (d == 3 && sys.is_pinned(s)) continue;
        double sd = std::sqrt(t / sys.masses[s]);
        for (int a = 0; a < d; a++)
            vel[d * i + a] = sys.to_step_displacement(sd * normal(seed, STREAM_VELOCITY, (uint32_t)d * (uint32_t)i + (uint32_t)a));
    }
    zero_velocity_sum(sys, species, vel, d == 3);
    return vel;
}
// init.rs:61-74 (2D): speed sqrt(2 t / m), direction TAU uniform(seed, 3, i), libm (fdlibm) cos
// and sin; then the zero velocity sum over every particle.
inline std::vector<int32_t> fixed_speed(const System& sys, const std::vector<uint32_t>& species, double t, uint64_t seed) {
    const size_t n = species.size();
    std::vector<int32_t> vel(2 * n, 0);
    for (size_t i = 0; i < n; i++) {
        const double speed = std::sqrt(2.0 * t / sys.masses[species[i]]);
        const double th = 6.28318530717958647692 * uniform(seed, 3, (uint32_t)i);
        vel[2 * i] = sys.to_step_displacement(speed * fdlibm::cos(th));
        vel[2 * i + 1] = sys.to_step_displacement(speed * fdlibm::sin(th));
    }
    zero_velocity_sum(sys, species, vel, false);
    return vel;
}
// init.rs:223-260 (2D): heights from the barometric law between margin and L_y - margin, x
// uniform, draws (stream 2 for x, 3 for y, one counter across attempts) rejected within min_sep
// of a placed particle (x periodic); positions only (the caller draws Maxwell velocities).
inline std::vector<int64_t> barometric_positions(const System& sys, const std::vector<uint32_t>& species, double t, double min_sep,
                                                 double margin, uint64_t seed) {
    const double b[2] = {sys.box_f64(0), sys.box_f64(1)};
    const double g = -sys.gravity[1];
    const double h = b[1] - 2.0 * margin;
    const double cell = std::max(min_sep, 0.5);
    const size_t gx = (size_t)std::ceil(b[0] / cell), gy = (size_t)std::ceil(b[1] / cell);
    std::vector<std::vector<size_t>> grid(gx * gy);
    std::vector<std::array<double, 2>> pos;
    uint32_t draw = 0;
    for (uint32_t s : species) {
        const double lam = sys.masses[s] * g / t;
        for (;;) {
            const double ux = uniform(seed, 2, draw), uy = uniform(seed, 3, draw);
            draw++;
            const double x = ux * b[0];
            const double y = margin + (lam > 1e-12 ? -std::log(1.0 - uy * (1.0 - std::exp(-lam * h))) / lam : uy * h);
            const size_t cx = std::min((size_t)(x / cell), gx - 1), cy = std::min((size_t)(y / cell), gy - 1);
            bool clash = false;
            for (size_t yy = cy > 0 ? cy - 1 : 0; yy < std::min(cy + 2, gy) && !clash; yy++)
                for (size_t ox = 0; ox < 3 && !clash; ox++) {
                    const size_t xx = (cx + gx + ox - 1) % gx;
                    for (size_t j : grid[yy * gx + xx]) {
                        double dx = std::fabs(pos[j][0] - x);
                        dx = std::min(dx, b[0] - dx);
                        const double dy = pos[j][1] - y;
                        if (dx * dx + dy * dy < min_sep * min_sep) {
                            clash = true;
                            break;
                        }
                    }
                }
            if (!clash) {
                grid[cy * gx + cx].push_back(pos.size());
                pos.push_back({x, y});
                break;
            }
        }
    }
    std::vector<int64_t> out(2 * pos.size());
    for (size_t i = 0; i < pos.size(); i++) {
        out[2 * i] = to_fixed(pos[i][0]);
        out[2 * i + 1] = to_fixed(pos[i][1]);
    }
    return out;
}
// init.rs:152-163: species of the particles within radius of center (min image, f64).
inline void mark_disc(const System& sys, State& s, const double* center, double radius, uint32_t species) {
    const int64_t c[2] = {to_fixed(center[0]), to_fixed(center[1])};
    const double r2 = radius * radius;
    for (size_t i = 0; i < s.n(); i++) {
        const double dx = to_f64(min_image(c[0], s.pos[2 * i], sys.box[0]));
        const double dy = to_f64(min_image(c[1], s.pos[2 * i + 1], sys.box[1]));
        if (dx * dx + dy * dy < r2) s.species[i] = species;
    }
}
// init.rs:105-121: on an axis with walls the lattice keeps 1 sigma clear of them.
inline State fluid(const System& sys, size_t n, double t, uint64_t seed) {
    State s;
    s.dim = 2;
    const int64_t margin = to_fixed(1.0);
    int64_t inner[2];
    for (int a = 0; a < 2; a++) inner[a] = sys.periodic(a) ? sys.box[a] : sys.box[a] - to_fixed(2.0);
    s.pos = lattice(n, {inner[0], inner[1]}, 0.1, seed);
    for (size_t i = 0; i < n; i++)
        for (int a = 0; a < 2; a++)
            if (!sys.periodic(a)) s.pos[2 * i + a] += margin;
    s.species.assign(n, 0);
    s.vel = maxwell(sys, s.species, t, seed);
    return s;
}
// init.rs:92-103 / three.rs:392-404: half-step kinetic temperature rescale.
inline double half_step_kinetic(const System& sys, const State& s) {
    double ke = 0.0;
    int d = sys.dim;
    for (size_t i = 0; i < s.n(); i++) {
        if (d == 3 && sys.is_pinned(s.species[i])) continue;
        double m = sys.masses[s.species[i]];
        if (d == 2) {
            double vx = sys.velocity(s.vel[2 * i]), vy = sys.velocity(s.vel[2 * i + 1]);
            ke += 0.5 * m * (vx * vx + vy * vy);
        } else {
            double acc = 0.0;
            for (int a = 0; a < 3; a++) acc += powi(sys.velocity(s.vel[3 * i + a]), 2);
            ke += 0.5 * m * acc;
        }
    }
    return ke;
}
inline void set_temperature(State& s, const System& sys, double t) {
    int d = sys.dim;
    size_t moving = 0;
    for (size_t i = 0; i < s.n(); i++)
        if (d == 2 || !sys.is_pinned(s.species[i])) moving++;
    double dof = d == 2 ? std::max((double)s.n() - 1.0, 1.0) : 1.5 * std::max((double)moving - 1.0, 1.0);
    double now = half_step_kinetic(sys, s) / dof;
    if (now <= 0.0) return;
    double f = std::sqrt(t / now);
    for (auto& v : s.vel) v = sat_i32(std::round((double)v * f));
    zero_velocity_sum(sys, s.species, s.vel, d == 3);
}

// three.rs:312-315
inline std::array<int64_t, 3> cube_for(size_t n, double density) {
    int64_t l = to_fixed(std::cbrt((double)n / density));
    return {l, l, l};
}
// three.rs:346-355
inline std::array<size_t, 3> fcc_cells(size_t n, std::array<int64_t, 3> box) {
    double b[3] = {to_f64(box[0]), to_f64(box[1]), to_f64(box[2])};
    double a = std::cbrt(b[0] * b[1] * b[2] * 4.0 / (double)n);
    std::array<size_t, 3> c;
    for (int k = 0; k < 3; k++) c[k] = std::max<size_t>((size_t)sat_u32(std::round(b[k] / a)), 1);
    while (4 * c[0] * c[1] * c[2] < n) {
        // the axis with the largest lattice constant (min_by of the reversed total order: the
        // first maximum)
        int k = 0;
        for (int x = 1; x < 3; x++)
            if (b[x] / (double)c[x] > b[k] / (double)c[k]) k = x;
        c[k]++;
    }
    return c;
}
// three.rs:319-343
inline std::vector<int64_t> fcc(size_t n, std::array<int64_t, 3> box, std::array<size_t, 3> cells, double jitter, uint64_t seed) {
    static const double basis[4][3] = {{0.25, 0.25, 0.25}, {0.75, 0.75, 0.25}, {0.75, 0.25, 0.75}, {0.25, 0.75, 0.75}};
    double a[3];
    for (int k = 0; k < 3; k++) a[k] = to_f64(box[k]) / (double)cells[k];
    std::vector<int64_t> out;
    out.reserve(3 * n);
    for (size_t k = 0; k < cells[2]; k++)
        for (size_t j = 0; j < cells[1]; j++)
            for (size_t i = 0; i < cells[0]; i++)
                for (int s = 0; s < 4; s++) {
                    if (out.size() / 3 == n) return out;
                    uint32_t id = (uint32_t)(out.size() / 3);
                    double cell[3] = {(double)i, (double)j, (double)k};
                    for (int ax = 0; ax < 3; ax++) {
                        double jit = jitter * (uniform(seed, STREAM_JITTER, 3 * id + (uint32_t)ax) - 0.5);
                        out.push_back(wrap(to_fixed((cell[ax] + basis[s][ax]) * a[ax] + jit), box[ax]));
                    }
                }
    return out;
}

// This engine's triangular-lattice start (no reference counterpart: md-core has a square-ish
// lattice and FCC only). Rows of spacing a = Lx / nx, odd rows shifted by a / 2, nx chosen so
// that the rows are as close to equilateral as the box allows, ny rounded up to an even number
// so the stacking is periodic; even rows at x = (i + 1/4) a, odd rows at (i + 3/4) a (so a slab
// of it keeps a quarter spacing clear of both its edges); the first n sites in row-major order,
// jittered like init::lattice (stream JITTER, counters 2k and 2k + 1).
inline void triangular_shape(size_t n, double b0, double b1, size_t* nx, size_t* ny) {
    size_t x = std::max<size_t>((size_t)sat_u32(std::round(std::sqrt((double)n * (b0 / b1) * 0.86602540378443864676))), 1);
    size_t y = (n + x - 1) / x;
    if (y > 1 && (y & 1)) y++;
    *nx = x;
    *ny = y;
}
inline std::vector<int64_t> triangular(size_t n, std::array<int64_t, 2> box, std::array<int64_t, 2> origin, std::array<int64_t, 2> wrap_len,
                                       double jitter, uint64_t seed, uint32_t first_id) {
    double b0 = to_f64(box[0]), b1 = to_f64(box[1]);
    size_t nx, ny;
    triangular_shape(n, b0, b1, &nx, &ny);
    double a0 = b0 / (double)nx, a1 = b1 / (double)ny;
    std::vector<int64_t> pos(2 * n);
    for (size_t k = 0; k < n; k++) {
        size_t i = k % nx, j = k / nx;
        uint32_t id = first_id + (uint32_t)k;
        double jx = jitter * (uniform(seed, STREAM_JITTER, 2 * id) - 0.5);
        double jy = jitter * (uniform(seed, STREAM_JITTER, 2 * id + 1) - 0.5);
        double shift = (j & 1) ? 0.75 : 0.25;
        pos[2 * k] = wrap(origin[0] + to_fixed(((double)i + shift) * a0 + jx), wrap_len[0]);
        pos[2 * k + 1] = wrap(origin[1] + to_fixed(((double)j + 0.5) * a1 + jy), wrap_len[1]);
    }
    return pos;
}

// This engine's liquid-vapour slab (no reference counterpart; md/tests/coexistence.rs:10-18
// builds its slab with init::fluid). The liquid fills x in [L (1 - f) / 2, L (1 + f) / 2) on a
// triangular lattice at rho_l; the vapour fills the rest of the box, 1 sigma clear of the
// liquid's edges, on a square lattice whose sites are displaced uniformly within
// (spacing - 1 sigma) so that no two vapour particles start closer than 1 sigma (stream VAPOUR,
// counters 2k, 2k + 1).
struct SlabShape {
    size_t n_liquid, n_vapour, vx, vy;
    int64_t x0, x1; // liquid region
};
inline SlabShape slab_shape(const System& sys, size_t n, double rho_l, double rho_v, double frac) {
    double lx = sys.box_f64(0), ly = sys.box_f64(1);
    SlabShape s;
    s.x0 = to_fixed(lx * (1.0 - frac) * 0.5);
    s.x1 = to_fixed(lx * (1.0 + frac) * 0.5);
    double wl = to_f64(s.x1 - s.x0);
    s.n_liquid = std::min(n, (size_t)sat_u32(std::round(rho_l * wl * ly)));
    s.n_vapour = n - s.n_liquid;
    double wv = std::max(lx - wl - 2.0, 0.0);
    // vapour lattice: vx columns over the vapour width, vy rows
    size_t vy = std::max<size_t>((size_t)sat_u32(std::ceil(std::sqrt((double)s.n_vapour * ly / std::max(wv, 1e-9)))), 1);
    size_t vx = s.n_vapour ? (s.n_vapour + vy - 1) / vy : 0;
    s.vx = vx;
    s.vy = vy;
    return s;
}
inline State slab(const System& sys, size_t n, double rho_l, double rho_v, double frac, double t, double jitter, uint64_t seed) {
    SlabShape sh = slab_shape(sys, n, rho_l, rho_v, frac);
    State st;
    st.dim = 2;
    st.pos.resize(2 * n);
    auto liq = triangular(sh.n_liquid, {sh.x1 - sh.x0, sys.box[1]}, {sh.x0, 0}, {sys.box[0], sys.box[1]}, jitter, seed, 0);
    std::copy(liq.begin(), liq.end(), st.pos.begin());
    double lx = sys.box_f64(0), ly = sys.box_f64(1);
    double wv = std::max(lx - to_f64(sh.x1 - sh.x0) - 2.0, 0.0);
    if (sh.n_vapour) {
        double ax = wv / (double)sh.vx, ay = ly / (double)sh.vy;
        double room_x = std::max(ax - 1.0, 0.0), room_y = std::max(ay - 1.0, 0.0);
        for (size_t k = 0; k < sh.n_vapour; k++) {
            size_t i = k % sh.vx, j = k / sh.vx;
            uint32_t c = (uint32_t)k;
            double ux = uniform(seed, STREAM_VAPOUR, 2 * c), uy = uniform(seed, STREAM_VAPOUR, 2 * c + 1);
            double x = (double)i * ax + 0.5 * (ax - room_x) + ux * room_x; // in the vapour strip
            double y = (double)j * ay + 0.5 * (ay - room_y) + uy * room_y;
            // the vapour strip starts 1 sigma past x1 and wraps around to 1 sigma before x0
            int64_t xf = wrap(sh.x1 + to_fixed(1.0 + x), sys.box[0]);
            size_t id = sh.n_liquid + k;
            st.pos[2 * id] = xf;
            st.pos[2 * id + 1] = wrap(to_fixed(y), sys.box[1]);
        }
    }
    st.species.assign(n, 0);
    st.vel = maxwell(sys, st.species, t, seed);
    return st;
}

// ---------------------------------------------------------------- md-ref/src/cells.rs
inline uint32_t cell_of(double x, double l, uint32_t n) { // cells.rs:53-55
    return std::min(sat_u32(x / l * (double)n), n - 1);
}
struct CellList { // cells.rs:1-32
    std::array<uint32_t, 3> dims{1, 1, 1};
    std::vector<uint32_t> keys, start, items;
};
// Row-major cell keys (2D: y nx + x; 3D: (z ny + y) nx + x) and a stable counting sort.
inline CellList build_cells(const System& sys, const State& s, std::array<uint32_t, 3> dims) {
    CellList cl;
    cl.dims = dims;
    int d = sys.dim;
    size_t n = s.n();
    uint32_t ncell = dims[0] * dims[1] * (d == 3 ? dims[2] : 1);
    cl.keys.resize(n);
    for (size_t i = 0; i < n; i++) {
        uint32_t c[3] = {0, 0, 0};
        for (int a = 0; a < d; a++) c[a] = cell_of(to_f64(s.pos[d * i + a]), sys.box_f64(a), dims[a]);
        cl.keys[i] = d == 2 ? c[1] * dims[0] + c[0] : (c[2] * dims[1] + c[1]) * dims[0] + c[0];
    }
    cl.start.assign(ncell + 1, 0);
    for (auto k : cl.keys) cl.start[k + 1]++;
    for (uint32_t c = 0; c < ncell; c++) cl.start[c + 1] += cl.start[c];
    std::vector<uint32_t> fill(cl.start.begin(), cl.start.end() - 1);
    cl.items.resize(n);
    for (size_t i = 0; i < n; i++) cl.items[fill[cl.keys[i]]++] = (uint32_t)i;
    return cl;
}

// ---------------------------------------------------------------- md-ref/src/real.rs
template <typename F> struct Real;
template <> struct Real<float> {
    static bool sep(int64_t d, float* o) { return sep_f32(d, o); }
    static float sep_near(int64_t d) { return sep_near_f32(d); }
    static float sep_long(int64_t d) { return sep_long_f32(d); } // real.rs:52-54
    static float from_f64(double x) { return (float)x; }
    static int32_t round_to_i32(float x) { return sat_i32f(std::rint(x)); }
    static constexpr bool is_f32 = true;
};
template <> struct Real<double> {
    static bool sep(int64_t d, double* o) {
        if (!(d >= -SEP_LIMIT && d < SEP_LIMIT)) return false;
        *o = to_f64(d);
        return true;
    }
    static double sep_near(int64_t d) { return to_f64(d); }
    static double sep_long(int64_t d) { return to_f64(d); } // real.rs:91-93
    static double from_f64(double x) { return x; }
    static int32_t round_to_i32(double x) { return sat_i32(std::rint(x)); }
    static constexpr bool is_f32 = false;
};
// md_core::BondType (system.rs:70-96) and md-ref's BondConsts (real.rs:161-197): the bond's
// -U'(r)/r and U at squared separation r2, in F, the reference's operation order.
struct BondType {
    bool fene = false; // else harmonic
    double k = 0.0, r0 = 0.0;
};
template <typename F> struct BondConsts {
    bool fene;
    F k, r0;
    static BondConsts make(const BondType& b) { return {b.fene, Real<F>::from_f64(b.k), Real<F>::from_f64(b.r0)}; }
    void eval(F r2, F* fr, F* u) const {
        const F one = Real<F>::from_f64(1.0), half = Real<F>::from_f64(0.5);
        if (fene) {
            F x = r2 / (r0 * r0);
            const F cap = Real<F>::from_f64(0.999999);
            if (x > cap) x = cap;
            *u = -half * k * r0 * r0 * Real<F>::from_f64(std::log((double)(one - x)));
            *fr = -k / (one - x);
        } else if (r0 == Real<F>::from_f64(0.0)) { // a zero-length spring (tethers): -k exactly
            *fr = -k;
            *u = half * k * r2;
        } else {
            const F r = std::sqrt(r2);
            const F dr = r - r0;
            *fr = -k * dr / r;
            *u = half * k * dr * dr;
        }
    }
};
constexpr uint32_t MAX_BONDS = 4; // system.rs:66

// real.rs:105-157
template <typename F> struct PairConsts {
    F rc2, eps4, sigma2, shift;
    F six_eps4; // 6 * eps4, the first product of eval's left-to-right chain
    static PairConsts make(const Pair& p) {
        PairConsts c;
        if (Real<F>::is_f32) { // pair.rs:54-56 gpu_constants, rounded once
            c.rc2 = (F)(float)(p.rc * p.rc);
            c.eps4 = (F)(float)(4.0 * p.eps);
            c.sigma2 = (F)(float)(p.sigma * p.sigma);
            c.shift = (F)(float)p.shift();
        } else {
            c.rc2 = (F)(p.rc * p.rc);
            c.eps4 = (F)(4.0 * p.eps);
            c.sigma2 = (F)(p.sigma * p.sigma);
            c.shift = (F)p.shift();
        }
        c.six_eps4 = (F)6.0 * c.eps4;
        return c;
    }
    // eval/eval3: r2 = fx fx + fy fy (+ fz fz); None unless r2 < rc2.
    bool eval(const F* f, int d, F* fr, F* u) const {
        F r2 = f[0] * f[0] + f[1] * f[1];
        if (d == 3) r2 = r2 + f[2] * f[2];
        if (!(r2 < rc2)) return false;
        F s2 = sigma2 / r2;
        F s6 = s2 * s2 * s2;
        *fr = (F)6.0 * eps4 * s6 * ((F)2.0 * s6 - (F)1.0) / r2;
        *u = eps4 * s6 * (s6 - (F)1.0) - shift;
        return true;
    }
};

// ---------------------------------------------------------------- md-core/src/table.rs
struct IntTables {
    static constexpr uint32_t SEP_BITS = 20, R2_BITS = 24, T_BITS = 2, KICK_SHIFT = 22, STEP_BITS = 12;
    size_t ns = 1, len = 0;
    std::vector<int32_t> data;
    std::vector<uint32_t> rc2;
    explicit IntTables(const System& sys) { // table.rs:45-71
        ns = (size_t)sys.species();
        double rcm = sys.rc_max();
        double rc2_max = rcm * rcm;
        len = (size_t)((uint64_t)(rc2_max * 16777216.0) >> STEP_BITS) + 2;
        data.assign(ns * ns * len, 0);
        rc2.assign(ns * ns, 0);
        for (size_t a = 0; a < ns; a++) {
            double c = sys.kick_coeff((uint32_t)a);
            for (size_t b = 0; b < ns; b++) {
                const Pair& p = sys.pair((uint32_t)a, (uint32_t)b);
                rc2[a * ns + b] = sat_u32(p.rc * p.rc * 16777216.0);
                Pair cont = p;
                cont.rc = INFINITY;
                for (size_t k = 0; k < len; k++) {
                    double r2 = (double)((uint64_t)k * 4096ull) / 16777216.0;
                    r2 = std::max(r2, 0.36);
                    double t = r2 < p.rc * p.rc + 2.0 * 4096.0 / 16777216.0 ? cont.f_over_r(r2) * c * 4.0 : 0.0;
                    double rt = std::round(t);
                    rt = std::min(std::max(rt, -2147483648.0), 2147483647.0);
                    data[(a * ns + b) * len + k] = sat_i32(rt);
                }
            }
        }
    }
    // table.rs:76-105 (2D)
    bool kick(uint32_t sa, uint32_t sb, const int64_t* d, int dim, int32_t* out) const {
        const int64_t limit = (int64_t)8 << 32;
        for (int a = 0; a < dim; a++)
            if (!(d[a] >= -limit && d[a] < limit)) return false;
        int64_t q[3] = {0, 0, 0};
        for (int a = 0; a < dim; a++) {
            uint64_t ax = d[a] < 0 ? (uint64_t)0 - (uint64_t)d[a] : (uint64_t)d[a];
            int64_t m = (int64_t)((ax + (1ull << (31 - SEP_BITS))) >> (32 - SEP_BITS));
            q[a] = d[a] < 0 ? -m : m;
        }
        uint64_t sq = 0;
        for (int a = 0; a < dim; a++) sq += (uint64_t)(q[a] * q[a]);
        uint32_t r2 = (uint32_t)((sq + (1ull << (2 * SEP_BITS - R2_BITS - 1))) >> (2 * SEP_BITS - R2_BITS));
        size_t pair = (size_t)sa * ns + sb;
        if (r2 >= rc2[pair]) return false;
        size_t idx = r2 >> STEP_BITS;
        int64_t frac = (int64_t)(r2 & ((1u << STEP_BITS) - 1));
        size_t base = pair * len;
        int64_t t0 = data[base + idx], t1 = data[base + idx + 1];
        int64_t t = t0 + (((t1 - t0) * frac) >> STEP_BITS);
        for (int a = 0; a < dim; a++) {
            unsigned __int128 prod = (unsigned __int128)(uint64_t)(t < 0 ? -t : t) * (unsigned __int128)(uint64_t)(q[a] < 0 ? -q[a] : q[a]);
            int64_t m = (int64_t)(uint64_t)(prod >> KICK_SHIFT);
            bool neg = (t < 0) != (q[a] < 0);
            out[a] = (int32_t)(neg ? m : -m);
        }
        return true;
    }
};

// ---------------------------------------------------------------- md-ref/src/fast.rs (2D)
// fast.rs:76-80
inline bool fast_eligible(const System& sys, std::array<uint32_t, 3> cells) {
    double side = std::max(sys.box_f64(0) / (double)cells[0], sys.box_f64(1) / (double)cells[1]);
    return 2.0 * side < 7.9;
}
template <typename F> struct FastScratch {
    std::vector<int64_t> sx, sy, nx, ny;
    std::vector<uint32_t> ss, sid, start, fill, key, ni;
    std::vector<int32_t> kx, ky, nkx, nky;
    std::vector<F> rx, ry;
};
// fast.rs:230-251
template <typename F>
inline void row_uniform(const PairConsts<F>& p, F c, size_t lo, size_t hi, size_t m, const F* rx, const F* ry, int32_t* tkx, int32_t* tky,
                        int32_t* okx, int32_t* oky, F* ope) {
    const F zero = (F)0, one = (F)1, two = (F)2, six = (F)6;
    int32_t kx = 0, ky = 0;
    F pe = zero;
    for (size_t k = 0; k < m; k++) {
        F x = rx[k], y = ry[k];
        F r2 = x * x + y * y;
        F s2 = p.sigma2 / r2;
        F s6 = s2 * s2 * s2;
        F f = six * p.eps4 * s6 * (two * s6 - one) / r2;
        F e = p.eps4 * s6 * (s6 - one) - p.shift;
        bool on = r2 < p.rc2 && k >= lo && k < hi;
        F a = -(on ? f : zero) * c;
        kx = wadd(kx, Real<F>::round_to_i32(a * x));
        ky = wadd(ky, Real<F>::round_to_i32(a * y));
        tkx[k] = wadd(tkx[k], Real<F>::round_to_i32(a * -x));
        tky[k] = wadd(tky[k], Real<F>::round_to_i32(a * -y));
        pe += on ? e : zero;
    }
    *okx = kx;
    *oky = ky;
    *ope = pe;
}
// fast.rs:257-294
template <typename F>
inline void row_mixture(const PairConsts<F>* row, const F* kick_c, size_t si, size_t lo, size_t hi, size_t m, const F* rx, const F* ry,
                        const uint32_t* ti, const uint32_t* species, int32_t* tkx, int32_t* tky, int32_t* okx, int32_t* oky, F* ope) {
    const F zero = (F)0, one = (F)1, two = (F)2, six = (F)6;
    F ci = kick_c[si];
    int32_t kx = 0, ky = 0;
    F pe = zero;
    for (size_t k = 0; k < m; k++) {
        size_t sj = species[ti[k]];
        const PairConsts<F>& p = row[sj];
        F x = rx[k], y = ry[k];
        F r2 = x * x + y * y;
        F s2 = p.sigma2 / r2;
        F s6 = s2 * s2 * s2;
        F f = six * p.eps4 * s6 * (two * s6 - one) / r2;
        F e = p.eps4 * s6 * (s6 - one) - p.shift;
        bool on = r2 < p.rc2 && k >= lo && k < hi;
        f = on ? f : zero;
        F ai = -f * ci, aj = -f * kick_c[sj];
        kx = wadd(kx, Real<F>::round_to_i32(ai * x));
        ky = wadd(ky, Real<F>::round_to_i32(ai * y));
        tkx[k] = wadd(tkx[k], Real<F>::round_to_i32(aj * -x));
        tky[k] = wadd(tky[k], Real<F>::round_to_i32(aj * -y));
        pe += on ? e : zero;
    }
    *okx = kx;
    *oky = ky;
    *ope = pe;
}
// fast.rs:83-222: counting sort into cells, half shell, branch-free rows, one scatter per cell.
template <typename F>
inline double pair_kicks_fast(const System& sys, const State& st, const std::vector<PairConsts<F>>& consts, const std::vector<F>& kick_c,
                              std::array<uint32_t, 3> cells, FastScratch<F>& sc, int32_t* kicks) {
    const size_t LANES = 8;
    size_t n = st.n();
    size_t ns = (size_t)sys.species();
    uint32_t cnx = cells[0], cny = cells[1];
    size_t ncell = (size_t)cnx * cny;
    double b0 = sys.box_f64(0), b1 = sys.box_f64(1);
    int64_t l[2] = {sys.box[0], sys.box[1]};
    sc.key.resize(n);
    for (size_t i = 0; i < n; i++) {
        uint32_t cx = cell_of(to_f64(st.pos[2 * i]), b0, cnx), cy = cell_of(to_f64(st.pos[2 * i + 1]), b1, cny);
        sc.key[i] = cy * cnx + cx;
    }
    sc.start.assign(ncell + 1, 0);
    for (auto k : sc.key) sc.start[k + 1]++;
    for (size_t c = 0; c < ncell; c++) sc.start[c + 1] += sc.start[c];
    sc.sx.assign(n, 0);
    sc.sy.assign(n, 0);
    sc.ss.assign(n, 0);
    sc.sid.assign(n, 0);
    sc.fill.assign(sc.start.begin(), sc.start.end());
    for (size_t i = 0; i < n; i++) {
        uint32_t k = sc.key[i];
        uint32_t s = sc.fill[k]++;
        sc.sx[s] = st.pos[2 * i];
        sc.sy[s] = st.pos[2 * i + 1];
        sc.ss[s] = st.species[i];
        sc.sid[s] = (uint32_t)i;
    }
    sc.kx.assign(n, 0);
    sc.ky.assign(n, 0);
    static const int SHELL[4][2] = {{1, 0}, {-1, 1}, {0, 1}, {1, 1}};
    F pe = (F)0;
    for (uint32_t cy = 0; cy < cny; cy++) {
        for (uint32_t cx = 0; cx < cnx; cx++) {
            size_t c = (size_t)cy * cnx + cx;
            size_t a0 = sc.start[c], a1 = sc.start[c + 1];
            if (a0 == a1) continue;
            sc.nx.clear();
            sc.ny.clear();
            sc.ni.clear();
            struct Range { size_t b0, b1; int64_t shx, shy; };
            Range ranges[5];
            size_t nr = 0;
            ranges[nr++] = {a0, a1, 0, 0};
            for (auto& o : SHELL) {
                int tx = (int)cx + o[0], ty = (int)cy + o[1];
                uint32_t dx, dy;
                int64_t shx = 0, shy = 0;
                if (tx < 0) { dx = (uint32_t)(tx + (int)cnx); shx = -l[0]; }
                else if (tx >= (int)cnx) { dx = (uint32_t)(tx - (int)cnx); shx = l[0]; }
                else dx = (uint32_t)tx;
                if (ty < 0) { dy = (uint32_t)(ty + (int)cny); shy = -l[1]; }
                else if (ty >= (int)cny) { dy = (uint32_t)(ty - (int)cny); shy = l[1]; }
                else dy = (uint32_t)ty;
                size_t d = (size_t)dy * cnx + dx;
                ranges[nr++] = {sc.start[d], sc.start[d + 1], shx, shy};
            }
            for (size_t r = 0; r < nr; r++) {
                for (size_t q = ranges[r].b0; q < ranges[r].b1; q++) {
                    sc.nx.push_back(sc.sx[q] + ranges[r].shx);
                    sc.ny.push_back(sc.sy[q] + ranges[r].shy);
                    sc.ni.push_back((uint32_t)q);
                }
            }
            size_t m = sc.nx.size();
            size_t mp = (m + LANES - 1) / LANES * LANES;
            int64_t lx = sc.nx[m - 1], ly = sc.ny[m - 1];
            uint32_t li = sc.ni[m - 1];
            sc.nx.resize(mp, lx);
            sc.ny.resize(mp, ly);
            sc.ni.resize(mp, li);
            sc.nkx.assign(mp, 0);
            sc.nky.assign(mp, 0);
            sc.rx.resize(mp);
            sc.ry.resize(mp);
            for (size_t p = 0; p < a1 - a0; p++) {
                size_t s = a0 + p;
                int64_t xs = sc.sx[s], ys = sc.sy[s];
                for (size_t k = 0; k < mp; k++) {
                    sc.rx[k] = Real<F>::sep_near(sc.nx[k] - xs);
                    sc.ry[k] = Real<F>::sep_near(sc.ny[k] - ys);
                }
                int32_t kx, ky;
                F e;
                if (ns == 1)
                    row_uniform<F>(consts[0], kick_c[0], p + 1, m, mp, sc.rx.data(), sc.ry.data(), sc.nkx.data(), sc.nky.data(), &kx, &ky, &e);
                else {
                    size_t si = sc.ss[s];
                    row_mixture<F>(&consts[si * ns], kick_c.data(), si, p + 1, m, mp, sc.rx.data(), sc.ry.data(), sc.ni.data(), sc.ss.data(),
                                   sc.nkx.data(), sc.nky.data(), &kx, &ky, &e);
                }
                sc.kx[s] = wadd(sc.kx[s], kx);
                sc.ky[s] = wadd(sc.ky[s], ky);
                pe += e;
            }
            for (size_t k = 0; k < m; k++) {
                size_t t = sc.ni[k];
                sc.kx[t] = wadd(sc.kx[t], sc.nkx[k]);
                sc.ky[t] = wadd(sc.ky[t], sc.nky[k]);
            }
        }
    }
    for (size_t s = 0; s < n; s++) {
        kicks[2 * sc.sid[s]] = sc.kx[s];
        kicks[2 * sc.sid[s] + 1] = sc.ky[s];
    }
    return (double)pe;
}

// ---------------------------------------------------------------- IntEngine<F> / IntEngine3<F>
struct Energy { double kinetic = 0.0, potential = 0.0; };

// ---------------------------------------------------------------- the Andersen bath
constexpr uint32_t STREAM_THERMO = 0x5448524du; // walls.rs:110
constexpr double TAU = 6.28318530717958647692;  // std::f64::consts::TAU

// walls::andersen (walls.rs:113-133) for 2D: acts_on (species, and the region along the bath's
// axis of the position before the drift) and then, with probability rate dt, the new velocity
// (sigma/tau, before the fan's drift); three::andersen (three.rs:247-265) for 3D: species and
// pinning, three components. Threefry on (id, clock) under the seed's thermostat key; ln, cos
// and sin are Rust's f64 methods, i.e. the platform libm (glibc), as here.
inline bool andersen(const System& sys, uint32_t id, uint32_t clock, uint32_t s, const int64_t* p, double* out) {
    const Bath& th = sys.bath;
    if (!th.on) return false;
    if (!((th.species >> s) & 1u)) return false;
    if (sys.dim == 2 && !(th.region[0] <= p[th.axis] && p[th.axis] < th.region[1])) return false;
    if (sys.dim == 3 && sys.is_pinned(s)) return false;
    const std::array<uint32_t, 2> key{(uint32_t)sys.seed, (uint32_t)(sys.seed >> 32) ^ STREAM_THERMO};
    const auto r = threefry2x32({id, clock}, key);
    if (to_unit_f64({r[0], 0}) >= th.rate * sys.dt) return false;
    const auto r2 = threefry2x32({id, clock}, {key[0], key[1] ^ 1u});
    const double sd = std::sqrt(th.t / sys.masses[s]);
    if (sys.dim == 2) {
        const double u1 = 1.0 - to_unit_f64({r[1], 0});
        const double u2 = to_unit_f64({r2[0], 0});
        const double rad = std::sqrt(-2.0 * std::log(u1));
        const double a = TAU * u2;
        out[0] = sd * rad * std::cos(a);
        out[1] = sd * rad * std::sin(a);
    } else {
        const auto r3 = threefry2x32({id, clock}, {key[0], key[1] ^ 2u});
        const double rad = std::sqrt(-2.0 * std::log(1.0 - to_unit_f64({r[1], 0})));
        const double a = TAU * to_unit_f64({r2[0], 0});
        const double rad3 = std::sqrt(-2.0 * std::log(1.0 - to_unit_f64({r3[0], 0})));
        const double a3 = TAU * to_unit_f64({r3[1], 0});
        out[0] = sd * rad * std::cos(a);
        out[1] = sd * rad * std::sin(a);
        out[2] = sd * rad3 * std::cos(a3);
    }
    return true;
}

// walls::Ledger (walls.rs:40-50): per slot (2 axis + side for walls, 6 the bath) the energy given
// to the system and the normal momentum it gave the wall, summed in f64 in particle order as
// IntEngine does, and the hits; for the bath also the events rounded to 2^-24 and summed as
// integers (the order-free total the GPU engine keeps).
constexpr int LEDGER_SLOTS = 7, LEDGER_BATH = 6, MEMBRANE_LOW = 4, MEMBRANE_HIGH = 5; // walls.rs:7-14
struct Ledger {
    double energy[LEDGER_SLOTS] = {0, 0, 0, 0, 0, 0, 0};
    double impulse[LEDGER_SLOTS] = {0, 0, 0, 0, 0, 0, 0};
    uint64_t hits[LEDGER_SLOTS] = {0, 0, 0, 0, 0, 0, 0};
    int64_t bath_energy_fixed = 0;
    // every event's energy change and impulse also rounded to 2^-24 and summed as integers (the
    // order-free totals a parallel engine can reproduce exactly)
    int64_t energy_fixed[LEDGER_SLOTS] = {0, 0, 0, 0, 0, 0, 0};
    int64_t impulse_fixed[LEDGER_SLOTS] = {0, 0, 0, 0, 0, 0, 0};
};

constexpr uint32_t STREAM_WALL = 0x57414c4cu; // walls.rs:86
constexpr double SOFT_RC = 1.122462048309373;  // walls.rs:104, 2^(1/6)

// walls::mirror (walls.rs:28-38): a coordinate that left [0, l) mirrored back about -1/2 or
// l - 1/2 (an exact involution on integers); side 0 or 1, or -1 when inside.
inline int mirror(int64_t& x, int64_t l) {
    if (x < 0) {
        x = -1 - x;
        return 0;
    }
    if (x >= l) {
        x = 2 * l - 1 - x;
        return 1;
    }
    return -1;
}

// A thermal wall's new velocity: walls::thermal_velocity (walls.rs:89-101) in 2D, the normal
// component and one tangential; three::thermal_velocity (three.rs:222-243) in 3D, two tangential.
inline void thermal_velocity(const System& sys, uint32_t id, uint32_t clock, double t, double m, double inward, double* normal,
                             double* tang) {
    const std::array<uint32_t, 2> key{(uint32_t)sys.seed, (uint32_t)(sys.seed >> 32) ^ STREAM_WALL};
    const auto r = threefry2x32({id, clock}, key);
    const auto r2 = threefry2x32({id, clock}, {key[0], key[1] ^ 1u});
    const double u1 = 1.0 - to_unit_f64(r);
    const double u2 = 1.0 - to_unit_f64({r2[0], 0}), u3 = to_unit_f64({r2[1], 0});
    const double sd = std::sqrt(t / m);
    *normal = inward * sd * std::sqrt(-2.0 * std::log(u1));
    if (sys.dim == 2) {
        tang[0] = sd * std::sqrt(-2.0 * std::log(u2)) * std::cos(TAU * u3);
    } else {
        const double rad = sd * std::sqrt(-2.0 * std::log(u2));
        const double a = TAU * u3;
        tang[0] = rad * std::cos(a);
        tang[1] = rad * std::sin(a);
    }
}
inline int64_t ledger_fixed(double de) { return (int64_t)std::round(de * 16777216.0); }

// md-ref int_engine.rs:23-447 and int_engine3.rs:12-240: periodic or walled (hard, soft,
// thermal) boxes, an optional Andersen bath, the ledger, and in 2D bonds, membranes,
// compartments and the piston. One template serves 2D and 3D; in 2D `fast` selects fast.rs's half-shell path when it applies, as IntEngine::forces does.
template <typename F> struct IntEngine {
    System sys;
    State state;
    std::vector<PairConsts<F>> consts;
    std::vector<F> kick_c;
    std::array<int32_t, 3> gravity{0, 0, 0};
    std::array<uint32_t, 3> cells{1, 1, 1};
    int64_t steps = 0;
    uint32_t clock = 0;
    Ledger ledger;
    std::vector<std::array<double, 6>> wall_force; // per particle, the soft walls' forces (last forces())
    bool fast = true;
    IntTables* tables = nullptr;
    FastScratch<F> scratch;
    int threads = 1; // OpenMP threads for the 3D/2D reference loop (the CPU baseline)
    // Bonds (2D; md-ref int_engine.rs:27-29, 55-56): per particle id its partners' ids and bond
    // types (System::partner_table, system.rs:311-324), padded with UINT32_MAX.
    std::vector<BondConsts<F>> bond_consts;
    std::vector<std::array<uint32_t, 2 * MAX_BONDS>> partners;
    // The piston (2D; int_engine.rs:40-44, 61-69; system.rs:100-116, 274-282): a soft wall that
    // replaces the top of y at height piston_w (position units) and moves piston_v per step,
    // driven at a set speed (drive 1) or free (drive 2) under the gas and an external force
    // pushing down; it stops at [piston_lo, piston_hi]. piston_work is the gas's work on it
    // and piston_force the gas's force in the last forces() (eps/sigma, summed in 2^-16 units).
    int piston_drive = 0;
    double piston_mass = 0.0, piston_ext = 0.0;
    int64_t piston_w = 0, piston_lo = 0, piston_hi = 0;
    int32_t piston_v = 0;
    double piston_work = 0.0, piston_force = 0.0;

    // walls::CompartmentLedger (walls.rs:52-72; IntEngine::compartment_ledger, int_engine.rs:
    // 30-32): per slot and per compartment along the wall (compartment_of along the other axis,
    // 0 for the bath), each event rounded to 2^-24 and summed as integers, with the hits.
    uint32_t per_wall = 1;
    std::vector<int64_t> comp_energy_fixed, comp_impulse_fixed;
    std::vector<uint64_t> comp_hits;
    size_t comp_slot(int w, int axis, const int64_t* x) const {
        int64_t c = 0;
        if (sys.dim == 2 && axis < 2) {
            const int o = 1 - axis;
            if (sys.compartments[o]) c = x[o] >> sys.compartments[o];
        }
        return (size_t)w * per_wall + (size_t)c;
    }

    IntEngine(const System& s, const State& st) : state(st) {
        set_system(s);
        // System::compartment_counts (system.rs:247-250): the most along either axis
        for (int a = 0; a < 2 && sys.dim == 2; a++)
            if (sys.compartments[a]) per_wall = std::max<uint32_t>(per_wall, (uint32_t)(sys.box[a] >> sys.compartments[a]));
        comp_energy_fixed.assign((size_t)LEDGER_SLOTS * per_wall, 0);
        comp_impulse_fixed.assign((size_t)LEDGER_SLOTS * per_wall, 0);
        comp_hits.assign((size_t)LEDGER_SLOTS * per_wall, 0);
    }
    // System::with_bonds (system.rs:284-299) and the engine's partner table.
    void set_bonds(const std::vector<BondType>& types, const std::vector<std::array<uint32_t, 3>>& bonds) {
        bond_consts.clear();
        for (auto& t : types) bond_consts.push_back(BondConsts<F>::make(t));
        partners.assign(bonds.empty() ? 0 : state.n(), {});
        for (auto& p : partners) p.fill(UINT32_MAX);
        std::vector<uint32_t> used(state.n(), 0);
        for (auto& b : bonds)
            for (int e = 0; e < 2; e++) {
                const uint32_t me = e ? b[1] : b[0], other = e ? b[0] : b[1];
                const uint32_t k = used[me]++;
                partners[me][2 * k] = other;
                partners[me][2 * k + 1] = b[2];
            }
    }
    // System::with_piston (system.rs:274-282) and the engine's piston state (int_engine.rs:61-69).
    bool set_piston(int drive, double speed, double mass, double force, double start, double min) {
        if (drive == 0) {
            piston_drive = 0;
            return true;
        }
        const double max = sys.box_f64(1);
        if (sys.dim != 2 || sys.periodic(1) || drive < 1 || drive > 2 || !(start <= max && min < start) || (drive == 2 && !(mass > 0.0)))
            return false;
        piston_drive = drive;
        piston_mass = mass;
        piston_ext = force;
        piston_w = to_fixed(start);
        piston_v = drive == 1 ? sys.to_step_displacement(speed) : 0;
        piston_lo = to_fixed(min);
        piston_hi = to_fixed(max);
        piston_work = 0.0;
        return true;
    }
    // walls::piston_kick (walls.rs:143-146): the integer kick on a free piston for a net upward
    // force, F dt^2 / M in position units, rounded half away from zero.
    int32_t piston_kick(double net) const { return sat_i32(std::round(net * sys.dt * sys.dt / piston_mass * 4294967296.0)); }
    // IntEngine::move_piston (int_engine.rs:346-361): a free piston's kick, the drift, the stops.
    void move_piston(double gas_force) {
        if (!piston_drive) return;
        if (piston_drive == 2) piston_v = wadd(piston_v, piston_kick(gas_force - piston_ext));
        const int64_t old = piston_w;
        piston_w += (int64_t)piston_v;
        if (piston_w < piston_lo || piston_w > piston_hi) {
            piston_w = std::clamp(piston_w, piston_lo, piston_hi);
            piston_v = 0;
        }
        piston_work += gas_force * to_f64(piston_w - old);
    }
    // The constructor's derived constants; alone, a run-time change of system (GpuEngine::
    // update_system, engine.rs:895-934) that keeps the state, counters, clock and ledger.
    void set_system(const System& s) {
        sys = s;
        consts.clear();
        kick_c.clear();
        for (auto& p : sys.pairs) consts.push_back(PairConsts<F>::make(p));
        for (int k = 0; k < sys.species(); k++) kick_c.push_back(Real<F>::from_f64(sys.kick_coeff((uint32_t)k)));
        gravity = sys.gravity_kick();
        cells = sys.cells_for(sys.rc_max());
        if (tables) use_integer_tables();
    }
    ~IntEngine() { delete tables; }
    void use_integer_tables() { // IntEngine::integer (int_engine.rs:94-98)
        delete tables;
        tables = new IntTables(sys);
    }
    // 2D: present_cells (int_engine.rs:108-116)
    std::array<uint32_t, 3> present_cells() const {
        if (sys.dim == 3) return cells;
        uint32_t present = 0;
        for (auto s : state.species) present |= 1u << s;
        double rc = 0.0;
        int ns = sys.species();
        for (int a = 0; a < ns; a++)
            for (int b = 0; b < ns; b++)
                if ((present >> a & 1) && (present >> b & 1)) rc = std::max(rc, sys.pairs[a * ns + b].rc);
        if (rc <= 0.0) return cells;
        auto c = sys.cells_for(rc);
        return {std::max(c[0], cells[0]), std::max(c[1], cells[1]), 1};
    }

    // The kick on particle i and its share of the potential energy: the body of the reference
    // loop over the 3^d neighbouring cells (int_engine.rs:144-243 / int_engine3.rs:56-128), with
    // the soft walls' forces on i added into wf.
    void force_on(size_t i, const CellList& cl, const uint32_t* nc, const double* b, int32_t* kout, double* pe_out, double* wf,
                  int64_t* piston_out) const {
        int d = sys.dim;
        int ns = sys.species();
        const int64_t* pi = &state.pos[d * i];
        uint32_t si = state.species[i];
        F c = kick_c[si];
        uint32_t cc[3] = {0, 0, 0};
        for (int a = 0; a < d; a++) cc[a] = cell_of(to_f64(pi[a]), b[a], nc[a]);
        int32_t k[3] = {0, 0, 0};
        F pe_i = (F)0;
        double pe_i64 = 0.0;
        int oz_n = d == 3 ? 3 : 1;
        for (int oz = 0; oz < oz_n; oz++) {
            uint32_t z = d == 3 ? (cc[2] + nc[2] + (uint32_t)oz - 1) % nc[2] : 0;
            for (int oy = 0; oy < 3; oy++) {
                uint32_t y = (cc[1] + nc[1] + (uint32_t)oy - 1) % nc[1];
                for (int ox = 0; ox < 3; ox++) {
                    uint32_t x = (cc[0] + nc[0] + (uint32_t)ox - 1) % nc[0];
                    uint32_t cell = (z * nc[1] + y) * nc[0] + x;
                    for (uint32_t q = cl.start[cell]; q < cl.start[cell + 1]; q++) {
                        size_t j = cl.items[q];
                        if (j == i) continue;
                        const int64_t* pj = &state.pos[d * j];
                        if (!sys.interact_across(pi, pj)) continue; // int_engine.rs:161-163
                        int64_t dd[3];
                        for (int a = 0; a < d; a++) dd[a] = sys.periodic(a) ? min_image(pi[a], pj[a], sys.box[a]) : pj[a] - pi[a]; // int_engine.rs:118-120
                        if (tables) {
                            int32_t kk[3];
                            if (tables->kick(si, state.species[j], dd, d, kk)) {
                                for (int a = 0; a < d; a++) k[a] = wadd(k[a], kk[a]);
                                double r2 = 0.0;
                                for (int a = 0; a < d; a++) r2 += to_f64(dd[a]) * to_f64(dd[a]);
                                pe_i64 += sys.pair(si, state.species[j]).energy(r2);
                            }
                            continue;
                        }
                        F f[3];
                        bool ok = true;
                        for (int a = 0; a < d; a++) ok = ok && Real<F>::sep(dd[a], &f[a]);
                        if (!ok) continue;
                        F fr, u;
                        if (consts[si * ns + state.species[j]].eval(f, d, &fr, &u)) {
                            F aa = -fr * c;
                            for (int a = 0; a < d; a++) k[a] = wadd(k[a], Real<F>::round_to_i32(aa * f[a]));
                            pe_i += u;
                        }
                    }
                }
            }
        }
        // bonds (int_engine.rs:185-202): rounded per bond like pairs, separations by sep_long
        double bond_part = 0.0;
        if (!partners.empty()) {
            F bond_pe = (F)0;
            for (uint32_t q = 0; q < MAX_BONDS; q++) {
                const uint32_t j = partners[i][2 * q];
                if (j == UINT32_MAX) break;
                const BondConsts<F>& bc = bond_consts[partners[i][2 * q + 1]];
                const int64_t* pj = &state.pos[d * j];
                F f[3] = {(F)0, (F)0, (F)0};
                for (int a = 0; a < d; a++) f[a] = Real<F>::sep_long(sys.periodic(a) ? min_image(pi[a], pj[a], sys.box[a]) : pj[a] - pi[a]);
                F r2 = f[0] * f[0] + f[1] * f[1];
                if (d == 3) r2 = r2 + f[2] * f[2];
                F fr, u;
                bc.eval(r2, &fr, &u);
                const F aa = -fr * c;
                for (int a = 0; a < d; a++) k[a] = wadd(k[a], Real<F>::round_to_i32(aa * f[a]));
                bond_pe += u;
            }
            bond_part = 0.5 * (double)bond_pe;
        }
        // soft walls (int_engine.rs:203-227, int_engine3.rs:107-126): WCA in the distance to
        // the wall, in F, its kick rounded like a pair's
        double wall_pe = 0.0;
        for (int a = 0; a < d; a++) {
            if (sys.periodic(a)) continue;
            for (int side = 0; side < 2; side++) {
                if (sys.wall_kind[a][side] != GBMD_WALL_SOFT) continue;
                const int64_t dw = side == 0 ? pi[a] : sys.box[a] - pi[a];
                F df;
                if (!Real<F>::sep(dw, &df)) continue;
                if (df < Real<F>::from_f64(SOFT_RC)) {
                    const F one = Real<F>::from_f64(1.0);
                    const F s2 = one / (df * df);
                    const F s6 = s2 * s2 * s2;
                    const F f = Real<F>::from_f64(24.0) * s6 * (Real<F>::from_f64(2.0) * s6 - one) / df;
                    const int32_t kw = Real<F>::round_to_i32(f * c);
                    k[a] = wadd(k[a], side == 0 ? kw : wneg(kw));
                    wf[2 * a + side] += (double)f;
                    wall_pe += (double)(Real<F>::from_f64(4.0) * s6 * (s6 - one) + one);
                }
            }
        }
        // the piston (int_engine.rs:230-246): a soft wall at piston_w pushing down; its force
        // summed in 2^-16 eps/sigma units (walls::PISTON_FORCE_SCALE, walls.rs:140-141)
        F df;
        if (piston_drive && Real<F>::sep(piston_w - pi[1], &df) && df < Real<F>::from_f64(SOFT_RC)) {
            const F one = Real<F>::from_f64(1.0);
            const F s2 = one / (df * df);
            const F s6 = s2 * s2 * s2;
            const F f = Real<F>::from_f64(24.0) * s6 * (Real<F>::from_f64(2.0) * s6 - one) / df;
            k[1] = wadd(k[1], wneg(Real<F>::round_to_i32(f * c)));
            *piston_out = sat_i64(std::round((double)f * 65536.0));
            wall_pe += (double)(Real<F>::from_f64(4.0) * s6 * (s6 - one) + one);
        }
        for (int a = 0; a < d; a++) kout[a] = k[a];
        *pe_out = bond_part + (tables ? 0.5 * pe_i64 : 0.5 * (double)pe_i) + wall_pe;
    }

    // A half shell for the 3D pair loop (the CPU baseline's form, off unless `half3` is set): each
    // pair in reach is evaluated once, from the particle earlier in cell order (the same cell after
    // it, and 13 of the 26 neighbouring cells), and each side's kick is rounded as the reference
    // loop rounds it: i gets round(-fr c_i f), j round(-fr c_j (-f)), with f = sep(min_image(x_i,
    // x_j)). j's own separation in the loop is exactly -f (min_image and sep are antisymmetric away
    // from half the box and from 8 sigma, both beyond every cutoff when the box holds three cells a
    // side), and r2 and fr are the same for both, so the kicks equal the loop's bit for bit in any
    // order of the wrapping integer sums. The potential is summed in f64 over pairs (its rounding
    // differs from the loop's per-particle f32 sums). Periodic pair systems, symmetric pair table.
    bool half3 = false;
    bool half3_ok(const std::array<uint32_t, 3>& nc) const {
        if (sys.dim != 3 || tables || !partners.empty() || !sys.all_periodic() || piston_drive) return false;
        for (int a = 0; a < 3; a++)
            if (nc[a] < 3) return false;
        const int ns = sys.species();
        for (int a = 0; a < ns; a++)
            for (int b = 0; b < ns; b++) {
                const Pair &p = sys.pairs[a * ns + b], &q = sys.pairs[b * ns + a];
                if (p.eps != q.eps || p.sigma != q.sigma || p.rc != q.rc) return false;
            }
        return true;
    }
    double forces_half3(std::vector<int32_t>& kicks, const std::array<uint32_t, 3>& dims) {
        const int ns = sys.species();
        CellList cl = build_cells(sys, state, dims);
        const uint32_t nc[3] = {dims[0], dims[1], dims[2]};
        uint32_t* ku = reinterpret_cast<uint32_t*>(kicks.data()); // wrapping sums (unsigned)
        static const int fwd[13][3] = {{1, 0, 0},  {-1, 1, 0}, {0, 1, 0},  {1, 1, 0},  {-1, -1, 1}, {0, -1, 1}, {1, -1, 1},
                                       {-1, 0, 1}, {0, 0, 1},  {1, 0, 1},  {-1, 1, 1}, {0, 1, 1},   {1, 1, 1}};
        const long long ncell = (long long)nc[0] * nc[1] * nc[2];
        double pe = 0.0;
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads) reduction(+ : pe) if (threads > 1)
        for (long long cc = 0; cc < ncell; cc++) {
            const uint32_t cell = (uint32_t)cc;
            const uint32_t cx = cell % nc[0], cy = (cell / nc[0]) % nc[1], cz = cell / (nc[0] * nc[1]);
            uint32_t nb[14];
            nb[0] = cell;
            for (int k = 0; k < 13; k++) {
                const uint32_t x = (cx + nc[0] + (uint32_t)(fwd[k][0] + 1) - 1) % nc[0];
                const uint32_t y = (cy + nc[1] + (uint32_t)(fwd[k][1] + 1) - 1) % nc[1];
                const uint32_t z = (cz + nc[2] + (uint32_t)(fwd[k][2] + 1) - 1) % nc[2];
                nb[k + 1] = (z * nc[1] + y) * nc[0] + x;
            }
            for (uint32_t p = cl.start[cell]; p < cl.start[cell + 1]; p++) {
                const size_t i = cl.items[p];
                const int64_t* pi = &state.pos[3 * i];
                const uint32_t si = state.species[i];
                const F ci = kick_c[si];
                int32_t k[3] = {0, 0, 0};
                for (int c = 0; c < 14; c++) {
                    const uint32_t q0 = c == 0 ? p + 1 : cl.start[nb[c]];
                    for (uint32_t q = q0; q < cl.start[nb[c] + 1]; q++) {
                        const size_t j = cl.items[q];
                        const int64_t* pj = &state.pos[3 * j];
                        F f[3];
                        bool ok = true;
                        for (int a = 0; a < 3; a++) ok = ok && Real<F>::sep(min_image(pi[a], pj[a], sys.box[a]), &f[a]);
                        if (!ok) continue;
                        const uint32_t sj = state.species[j];
                        F fr, u;
                        if (!consts[si * ns + sj].eval(f, 3, &fr, &u)) continue;
                        const F ai = -fr * ci, aj = -fr * kick_c[sj];
                        for (int a = 0; a < 3; a++) {
                            k[a] = wadd(k[a], Real<F>::round_to_i32(ai * f[a]));
                            const uint32_t kj = (uint32_t)Real<F>::round_to_i32(aj * (-f[a]));
#pragma omp atomic
                            ku[3 * j + a] += kj;
                        }
                        pe += (double)u;
                    }
                }
                for (int a = 0; a < 3; a++) {
                    const uint32_t ki = (uint32_t)k[a];
#pragma omp atomic
                    ku[3 * i + a] += ki;
                }
            }
        }
        piston_force = 0.0;
        return pe;
    }

    // IntEngine::forces (int_engine.rs:130-251) / IntEngine3::forces (int_engine3.rs:48-131):
    // the reference loop over the 3^d neighbouring cells of each particle, or the fast path.
    double forces(std::vector<int32_t>& kicks) {
        int d = sys.dim;
        size_t n = state.n();
        kicks.assign(d * n, 0);
        auto cl_dims = present_cells();
        double pe = 0.0;
        wall_force.assign(n, {0, 0, 0, 0, 0, 0});
        // (with walls the reference loop: fast.rs gives the same kicks, fast_path.rs:20-54)
        bool use_fast = d == 2 && fast && !tables && partners.empty() && sys.all_periodic() && fast_eligible(sys, cl_dims);
        if (use_fast) return pair_kicks_fast<F>(sys, state, consts, kick_c, cl_dims, scratch, kicks.data());
        if (half3 && half3_ok(cl_dims)) return forces_half3(kicks, cl_dims);
        CellList cl = build_cells(sys, state, cl_dims);
        uint32_t nc[3] = {cl_dims[0], cl_dims[1], d == 3 ? cl_dims[2] : 1u};
        double b[3] = {sys.box_f64(0), sys.box_f64(1), d == 3 ? sys.box_f64(2) : 1.0};
        std::vector<double> pe_part(n, 0.0);
        std::vector<int64_t> piston_part(n, 0);
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads) if (threads > 1)
        for (long long ii = 0; ii < (long long)n; ii++) {
            size_t i = (size_t)ii;
            force_on(i, cl, nc, b, &kicks[d * i], &pe_part[i], wall_force[i].data(), &piston_part[i]);
        }
        uint64_t piston_fixed = 0; // an integer sum (wrapping): the same in any order
        for (size_t i = 0; i < n; i++) {
            pe += pe_part[i];
            piston_fixed += (uint64_t)piston_part[i];
        }
        piston_force = (double)(int64_t)piston_fixed / 65536.0;
        return pe;
    }

    // The reference loop's kicks on the particles idx[0..m) only (what forces() gives them, the
    // fast path included, which equals the loop: fast_path.rs:20-54): a sample of a system too
    // large to evaluate whole within a test.
    void forces_of(const uint32_t* idx, size_t m, int32_t* out) const {
        int d = sys.dim;
        auto cl_dims = present_cells();
        CellList cl = build_cells(sys, state, cl_dims);
        uint32_t nc[3] = {cl_dims[0], cl_dims[1], d == 3 ? cl_dims[2] : 1u};
        double b[3] = {sys.box_f64(0), sys.box_f64(1), d == 3 ? sys.box_f64(2) : 1.0};
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads) if (threads > 1)
        for (long long q = 0; q < (long long)m; q++) {
            double pe_i, wf[6] = {0, 0, 0, 0, 0, 0};
            int64_t pf = 0;
            force_on(idx[q], cl, nc, b, out + d * q, &pe_i, wf, &pf);
        }
    }

    // int_engine.rs:253-344 / int_engine3.rs:138-184 (periodic): v += kick + g; the Andersen
    // bath (int_engine.rs:275-293, int_engine3.rs:155-160); x += v; wrap.
    void step(size_t nsteps) {
        int d = sys.dim;
        std::vector<int32_t> kicks;
        const int32_t drift = sys.to_step_displacement(sys.bath.drift);
        for (size_t s = 0; s < nsteps; s++) {
            forces(kicks);
            // the soft walls' impulses (int_engine.rs:256-263, int_engine3.rs:140-145)
            for (size_t i = 0; i < state.n(); i++)
                for (int w = 0; w < 6; w++)
                    if (wall_force[i][w] != 0.0) {
                        ledger.impulse[w] += wall_force[i][w] * sys.dt;
                        ledger.impulse_fixed[w] += ledger_fixed(wall_force[i][w] * sys.dt);
                        comp_impulse_fixed[comp_slot(w, w / 2, &state.pos[d * i])] += ledger_fixed(wall_force[i][w] * sys.dt);
                    }
            for (size_t i = 0; i < state.n(); i++) {
                const uint32_t sp = state.species[i];
                bool pinned = sys.is_pinned(sp);
                int32_t* v = &state.vel[d * i];
                int64_t* x = &state.pos[d * i];
                for (int a = 0; a < d; a++) v[a] = wadd(wadd(v[a], kicks[d * i + a]), pinned ? 0 : gravity[a]);
                double u[3] = {0.0, 0.0, 0.0};
                if (!pinned && andersen(sys, (uint32_t)i, clock, sp, x, u)) {
                    const double m = sys.masses[sp];
                    double de;
                    if (d == 2) {
                        const double b0 = sys.velocity(v[0]), b1 = sys.velocity(v[1]);
                        v[0] = wadd(sys.to_step_displacement(u[0]), drift);
                        v[1] = sys.to_step_displacement(u[1]);
                        if (piston_drive == 1) { // relative to the affine flow under a driven piston (int_engine.rs:282-286)
                            const double f = std::clamp(to_f64(x[1]) / to_f64(piston_w), 0.0, 1.0);
                            v[1] = wadd(v[1], sat_i32(std::round((double)piston_v * f)));
                        }
                        const double a0 = sys.velocity(v[0]), a1 = sys.velocity(v[1]);
                        de = 0.5 * m * (a0 * a0 + a1 * a1 - b0 * b0 - b1 * b1);
                    } else {
                        double before = 0.0, after = 0.0;
                        for (int a = 0; a < 3; a++) {
                            const double b = sys.velocity(v[a]);
                            before += b * b;
                        }
                        for (int a = 0; a < 3; a++) v[a] = sys.to_step_displacement(u[a]);
                        for (int a = 0; a < 3; a++) {
                            const double b = sys.velocity(v[a]);
                            after += b * b;
                        }
                        de = 0.5 * m * (after - before);
                    }
                    ledger.energy[LEDGER_BATH] += de;
                    ledger.bath_energy_fixed += ledger_fixed(de);
                    comp_energy_fixed[(size_t)LEDGER_BATH * per_wall] += ledger_fixed(de);
                    comp_hits[(size_t)LEDGER_BATH * per_wall] += 1;
                    ledger.hits[LEDGER_BATH] += 1;
                }
                int64_t old[3] = {x[0], x[1], d == 3 ? x[2] : 0};
                for (int a = 0; a < d; a++) x[a] += (int64_t)v[a];
                // the membrane (int_engine.rs:296-313): a blocked species outside a pore that
                // crossed it is mirrored about position - 1/2 (walls::cross_membrane, walls.rs:18-25)
                if (sys.membrane && d == 2 && sys.membrane_blocks_species(sp)) {
                    const int a = sys.membrane_axis;
                    const int64_t w = sys.membrane_position;
                    if (!sys.in_pore(old[1 - a]) && (old[a] < w) != (x[a] < w)) {
                        const int face = old[a] < w ? MEMBRANE_LOW : MEMBRANE_HIGH;
                        x[a] = 2 * w - 1 - x[a];
                        const double dp = 2.0 * sys.masses[sp] * std::fabs(sys.velocity(v[a]));
                        v[a] = wneg(v[a]);
                        ledger.impulse[face] += dp;
                        ledger.impulse_fixed[face] += ledger_fixed(dp);
                        comp_impulse_fixed[comp_slot(face, a, old)] += ledger_fixed(dp);
                        comp_hits[comp_slot(face, a, old)] += 1;
                        ledger.hits[face] += 1;
                    }
                }
                for (int a = 0; a < d; a++) {
                    if (sys.periodic(a)) {
                        x[a] = wrap(x[a], sys.box[a]);
                        continue;
                    }
                    const int side = mirror(x[a], sys.box[a]);
                    if (side >= 0) {
                        collide(i, a, side, v, old);
                    } else if (d == 2 && sys.compartments[a] != 0) {
                        // int_engine.rs:324-330: a particle that crossed into another compartment
                        // is mirrored back into its home one (walls::mirror_compartment, walls.rs:72-78)
                        const uint32_t sh = sys.compartments[a];
                        const int64_t home = old[a] >> sh;
                        if ((x[a] >> sh) != home) {
                            const int64_t lo = home << sh, hi = (home + 1) << sh;
                            x[a] = x[a] < lo ? 2 * lo - 1 - x[a] : (x[a] >= hi ? 2 * hi - 1 - x[a] : x[a]);
                            v[a] = wneg(v[a]);
                        }
                    }
                }
                if (piston_drive && x[1] >= piston_w) { // int_engine.rs:333-336: mirrored below the piston
                    x[1] = 2 * piston_w - 1 - x[1];
                    v[1] = wneg(v[1]);
                }
            }
            move_piston(piston_force);
            steps += 1;
            clock += 1;
        }
    }
    // IntEngine::collide (int_engine.rs:363-390) / IntEngine3::collide (int_engine3.rs:186-205):
    // hard and soft walls reflect the normal component; a thermal wall draws a new velocity; the
    // ledger books the energy change and the normal momentum given to the wall.
    void collide(size_t i, int axis, int side, int32_t* v, const int64_t* old) {
        const int d = sys.dim;
        const double m = sys.masses[state.species[i]];
        const int w = 2 * axis + side;
        double before[3] = {0, 0, 0}, after[3] = {0, 0, 0};
        for (int a = 0; a < d; a++) before[a] = sys.velocity(v[a]);
        if (sys.wall_kind[axis][side] == GBMD_WALL_THERMAL) {
            double vn = 0.0, vt[2] = {0.0, 0.0};
            thermal_velocity(sys, (uint32_t)i, clock, sys.wall_t[axis][side], m, side == 0 ? 1.0 : -1.0, &vn, vt);
            v[axis] = sys.to_step_displacement(vn);
            if (d == 2) {
                v[1 - axis] = sys.to_step_displacement(vt[0]);
            } else {
                v[(axis + 1) % 3] = sys.to_step_displacement(vt[0]);
                v[(axis + 2) % 3] = sys.to_step_displacement(vt[1]);
            }
        } else {
            v[axis] = wneg(v[axis]);
        }
        for (int a = 0; a < d; a++) after[a] = sys.velocity(v[a]);
        auto ke = [&](const double* u) { return d == 2 ? 0.5 * m * (u[0] * u[0] + u[1] * u[1]) : 0.5 * m * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]); };
        const double de = ke(after) - ke(before), imp = std::fabs(m * (before[axis] - after[axis]));
        ledger.energy[w] += de;
        ledger.impulse[w] += imp;
        ledger.energy_fixed[w] += ledger_fixed(de);
        ledger.impulse_fixed[w] += ledger_fixed(imp);
        ledger.hits[w] += 1;
        const size_t q = comp_slot(w, axis, old); // (the position before the move, as the reference's)
        comp_energy_fixed[q] += ledger_fixed(de);
        comp_impulse_fixed[q] += ledger_fixed(imp);
        comp_hits[q] += 1;
    }
    // int_engine.rs:396-413
    void reverse() {
        int d = sys.dim;
        std::vector<int32_t> kicks;
        forces(kicks);
        for (size_t i = 0; i < state.n(); i++) {
            bool pinned = sys.is_pinned(state.species[i]);
            for (int a = 0; a < d; a++) {
                int32_t g = pinned ? 0 : gravity[a];
                state.vel[d * i + a] = wneg(wadd(wadd(state.vel[d * i + a], kicks[d * i + a]), g));
            }
        }
        if (piston_drive) { // int_engine.rs:404-410
            const int32_t kick = piston_drive == 2 ? piston_kick(piston_force - piston_ext) : 0;
            piston_v = wneg(wadd(piston_v, kick));
        }
        steps = -steps;
    }
    // int_engine.rs:417-446 / int_engine3.rs:222-239: on-step KE and the potential energy.
    Energy energy() {
        int d = sys.dim;
        std::vector<int32_t> kicks;
        Energy e;
        e.potential = forces(kicks);
        for (size_t i = 0; i < state.n(); i++) {
            uint32_t s = state.species[i];
            if (d == 3 && sys.is_pinned(s)) continue;
            double m = sys.masses[s];
            if (d == 2) {
                double v[2];
                for (int a = 0; a < 2; a++) {
                    int32_t next = wadd(wadd(state.vel[2 * i + a], kicks[2 * i + a]), gravity[a]);
                    v[a] = 0.5 * (sys.velocity(state.vel[2 * i + a]) + sys.velocity(next));
                }
                e.kinetic += 0.5 * m * (v[0] * v[0] + v[1] * v[1]);
                for (int a = 0; a < 2; a++) e.potential -= m * sys.gravity[a] * to_f64(state.pos[2 * i + a]);
            } else {
                for (int a = 0; a < 3; a++) {
                    int32_t next = wadd(wadd(state.vel[3 * i + a], kicks[3 * i + a]), gravity[a]);
                    double v = 0.5 * (sys.velocity(state.vel[3 * i + a]) + sys.velocity(next));
                    e.kinetic += 0.5 * m * v * v;
                    e.potential -= m * sys.gravity[a] * to_f64(state.pos[3 * i + a]);
                }
            }
        }
        return e;
    }
};

// ---------------------------------------------------------------- md-ref/src/float_engine.rs
// FloatEngine<f64> in 2D (periodic): conventional MD in floats, the reference for observables.
struct FloatEngine {
    System sys;
    std::vector<double> pos, vel;
    std::vector<uint32_t> species;
    std::vector<PairConsts<double>> consts;
    double box[2];
    std::vector<double> inv_mass;
    std::array<uint32_t, 3> cells;
    FloatEngine(const System& s, const State& st) : sys(s) {
        box[0] = sys.box_f64(0);
        box[1] = sys.box_f64(1);
        for (size_t i = 0; i < st.n(); i++) {
            pos.push_back(to_f64(st.pos[2 * i]));
            pos.push_back(to_f64(st.pos[2 * i + 1]));
            vel.push_back(sys.velocity(st.vel[2 * i]));
            vel.push_back(sys.velocity(st.vel[2 * i + 1]));
        }
        species = st.species;
        for (auto& p : sys.pairs) consts.push_back(PairConsts<double>::make(p));
        for (double m : sys.masses) inv_mass.push_back(1.0 / m);
        cells = sys.cells_for(sys.rc_max());
    }
    double min_image_f(double d, int a) const {
        double l = box[a], half = l * 0.5;
        if (d >= half) return d - l;
        if (d < -half) return d + l;
        return d;
    }
    double forces(std::vector<double>& f) const {
        size_t n = species.size();
        int ns = sys.species();
        f.assign(2 * n, 0.0);
        uint32_t nc[2] = {cells[0], cells[1]};
        std::vector<uint32_t> keys(n);
        auto cellc = [&](size_t i, int a) { return cell_of(pos[2 * i + a], box[a], nc[a]); };
        for (size_t i = 0; i < n; i++) keys[i] = cellc(i, 1) * nc[0] + cellc(i, 0);
        std::vector<uint32_t> start(nc[0] * nc[1] + 1, 0), items(n);
        for (auto k : keys) start[k + 1]++;
        for (size_t c = 0; c + 1 < start.size(); c++) start[c + 1] += start[c];
        std::vector<uint32_t> fill(start.begin(), start.end() - 1);
        for (size_t i = 0; i < n; i++) items[fill[keys[i]]++] = (uint32_t)i;
        double pe = 0.0;
        for (size_t i = 0; i < n; i++) {
            uint32_t cx = cellc(i, 0), cy = cellc(i, 1);
            double fx_i = 0, fy_i = 0, pe_i = 0;
            for (int oy = 0; oy < 3; oy++) {
                uint32_t y = (cy + nc[1] + (uint32_t)oy - 1) % nc[1];
                for (int ox = 0; ox < 3; ox++) {
                    uint32_t x = (cx + nc[0] + (uint32_t)ox - 1) % nc[0];
                    uint32_t k = y * nc[0] + x;
                    for (uint32_t q = start[k]; q < start[k + 1]; q++) {
                        size_t j = items[q];
                        if (j == i) continue;
                        double dd[2] = {min_image_f(pos[2 * j] - pos[2 * i], 0), min_image_f(pos[2 * j + 1] - pos[2 * i + 1], 1)};
                        double fr, u;
                        if (consts[species[i] * ns + species[j]].eval(dd, 2, &fr, &u)) {
                            fx_i += -fr * dd[0];
                            fy_i += -fr * dd[1];
                            pe_i += u;
                        }
                    }
                }
            }
            f[2 * i] = fx_i;
            f[2 * i + 1] = fy_i;
            pe += 0.5 * pe_i;
        }
        return pe;
    }
    double wrapf(double x, int a) const { return x - box[a] * std::floor(x / box[a]); }
    void step(size_t nsteps) {
        std::vector<double> f;
        for (size_t s = 0; s < nsteps; s++) {
            forces(f);
            for (size_t i = 0; i < species.size(); i++) {
                double k = inv_mass[species[i]] * sys.dt;
                for (int a = 0; a < 2; a++) {
                    vel[2 * i + a] += f[2 * i + a] * k;
                    double x = pos[2 * i + a] + vel[2 * i + a] * sys.dt;
                    pos[2 * i + a] = wrapf(x, a);
                }
            }
        }
    }
    Energy energy() const {
        std::vector<double> f;
        Energy e;
        e.potential = forces(f);
        for (size_t i = 0; i < species.size(); i++) {
            double m = sys.masses[species[i]];
            double k = inv_mass[species[i]] * sys.dt;
            for (int a = 0; a < 2; a++) {
                double v = vel[2 * i + a] + 0.5 * f[2 * i + a] * k;
                e.kinetic += 0.5 * m * v * v;
            }
        }
        return e;
    }
};

// ---------------------------------------------------------------- Verlet lists (md shaders)
// neighbors.wgsl:27-64 / md3.wgsl:443-483 with an exactly specified f32 test: a pair is listed
// when the f32 separations (fixed.rs sep_f32; beyond 8 sigma the GPU's 1e30) give
// fx*fx + fy*fy (+ fz*fz), summed left to right without fusion, below the f32 of
// ((rc_ab + skin)(1 + 1e-4))^2 (engine.rs:302-313). Every listed pair is within the scanned
// 3^d cells because cells are at least rc + skin wide (engine.rs:152-153).
inline float pair_list_r2(const System& sys, uint32_t a, uint32_t b, double skin) {
    double r = (sys.pair(a, b).rc + skin) * (1.0 + 1e-4);
    return (float)(r * r);
}
inline float sep_or_far(int64_t d) {
    float f;
    return sep_f32(d, &f) ? f : 1e30f;
}
// The sorted indices of particle i's listed neighbours, from a cell list of the list radius.
inline std::vector<uint32_t> verlet_list_of(const System& sys, const State& s, const CellList& cl, const uint32_t* nc, size_t i, double skin) {
    int d = sys.dim;
    uint32_t key = cl.keys[i];
    uint32_t cc[3] = {key % nc[0], (key / nc[0]) % nc[1], key / (nc[0] * nc[1])};
    const int64_t* pi = &s.pos[d * i];
    std::vector<uint32_t> out;
    std::vector<uint32_t> seen;
    int oz_n = d == 3 ? 3 : 1;
    for (int oz = 0; oz < oz_n; oz++) {
        uint32_t z = d == 3 ? (cc[2] + nc[2] + (uint32_t)oz - 1) % nc[2] : 0;
        for (int oy = 0; oy < 3; oy++) {
            uint32_t y = (cc[1] + nc[1] + (uint32_t)oy - 1) % nc[1];
            for (int ox = 0; ox < 3; ox++) {
                uint32_t x = (cc[0] + nc[0] + (uint32_t)ox - 1) % nc[0];
                uint32_t cell = (z * nc[1] + y) * nc[0] + x;
                // a 3-cell-wide axis visits a cell once per offset; count each cell once
                if (std::find(seen.begin(), seen.end(), cell) != seen.end()) continue;
                seen.push_back(cell);
                for (uint32_t q = cl.start[cell]; q < cl.start[cell + 1]; q++) {
                    uint32_t j = cl.items[q];
                    if (j == i) continue;
                    const int64_t* pj = &s.pos[d * j];
                    float f[3] = {0.0f, 0.0f, 0.0f};
                    for (int a = 0; a < d; a++) f[a] = sep_or_far(sys.periodic(a) ? min_image(pi[a], pj[a], sys.box[a]) : pj[a] - pi[a]);
                    float r2 = f[0] * f[0] + f[1] * f[1];
                    if (d == 3) r2 = r2 + f[2] * f[2];
                    if (r2 < pair_list_r2(sys, s.species[i], s.species[j], skin)) out.push_back(j);
                }
            }
        }
    }
    std::sort(out.begin(), out.end());
    return out;
}
// Returns, for each particle (storage index), the sorted indices of its listed neighbours.
inline std::vector<std::vector<uint32_t>> verlet_lists(const System& sys, const State& s, double skin) {
    auto dims = sys.cells_for(sys.rc_max() + skin);
    CellList cl = build_cells(sys, s, dims);
    uint32_t nc[3] = {dims[0], dims[1], sys.dim == 3 ? dims[2] : 1u};
    std::vector<std::vector<uint32_t>> out(s.n());
    for (size_t i = 0; i < s.n(); i++) out[i] = verlet_list_of(sys, s, cl, nc, i, skin);
    return out;
}
// The lists of the particles idx[0..m) only (a sample of a system too large to list whole
// within a test), in parallel.
inline std::vector<std::vector<uint32_t>> verlet_lists_of(const System& sys, const State& s, double skin, const uint32_t* idx, size_t m,
                                                          int threads) {
    auto dims = sys.cells_for(sys.rc_max() + skin);
    CellList cl = build_cells(sys, s, dims);
    uint32_t nc[3] = {dims[0], dims[1], sys.dim == 3 ? dims[2] : 1u};
    std::vector<std::vector<uint32_t>> out(m);
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads) if (threads > 1)
    for (long long q = 0; q < (long long)m; q++) out[q] = verlet_list_of(sys, s, cl, nc, idx[q], skin);
    return out;
}
// ForceMode::verlet_with_skin (engine.rs:130-141) / verlet3_with_skin (engine3.rs:61-68),
// without the 128 MiB single-binding clamp (device memory has no per-binding cap here).
inline uint32_t verlet_cap(const System& sys, size_t n, double skin) {
    double r = sys.rc_max() + skin;
    double density = (double)n / sys.volume();
    double vol = sys.dim == 2 ? 3.14159265358979323846 * r * r : 4.0 / 3.0 * 3.14159265358979323846 * r * r * r;
    return sat_u32(std::ceil(vol * std::max(2.0 * density, 1.2))) + 8;
}

// ---------------------------------------------------------------- instruments (new)
// f32 pair terms exactly as the engine evaluates them, summed in f64: PE and the virial
// sum over pairs of fr r^2 (= -r dU/dr, mc/src/gibbs.rs:58-66), over unordered pairs.
struct PairSums { double potential = 0.0, virial = 0.0; };
inline PairSums pair_sums_f32(const System& sys, const State& s) {
    int d = sys.dim;
    int ns = sys.species();
    std::vector<PairConsts<float>> consts;
    for (auto& p : sys.pairs) consts.push_back(PairConsts<float>::make(p));
    auto dims = sys.cells_for(sys.rc_max());
    CellList cl = build_cells(sys, s, dims);
    uint32_t nc[3] = {dims[0], dims[1], d == 3 ? dims[2] : 1u};
    PairSums out;
    for (size_t i = 0; i < s.n(); i++) {
        uint32_t key = cl.keys[i];
        uint32_t cc[3] = {key % nc[0], (key / nc[0]) % nc[1], key / (nc[0] * nc[1])};
        const int64_t* pi = &s.pos[d * i];
        double pe_i = 0.0, w_i = 0.0;
        int oz_n = d == 3 ? 3 : 1;
        for (int oz = 0; oz < oz_n; oz++) {
            uint32_t z = d == 3 ? (cc[2] + nc[2] + (uint32_t)oz - 1) % nc[2] : 0;
            for (int oy = 0; oy < 3; oy++) {
                uint32_t y = (cc[1] + nc[1] + (uint32_t)oy - 1) % nc[1];
                for (int ox = 0; ox < 3; ox++) {
                    uint32_t x = (cc[0] + nc[0] + (uint32_t)ox - 1) % nc[0];
                    uint32_t cell = (z * nc[1] + y) * nc[0] + x;
                    for (uint32_t q = cl.start[cell]; q < cl.start[cell + 1]; q++) {
                        uint32_t j = cl.items[q];
                        if (j == i) continue;
                        const int64_t* pj = &s.pos[d * j];
                        float f[3];
                        bool ok = true;
                        for (int a = 0; a < d; a++)
                            ok = ok && sep_f32(sys.periodic(a) ? min_image(pi[a], pj[a], sys.box[a]) : pj[a] - pi[a], &f[a]);
                        if (!ok) continue;
                        float fr, u;
                        if (consts[s.species[i] * ns + s.species[j]].eval(f, d, &fr, &u)) {
                            float r2 = f[0] * f[0] + f[1] * f[1];
                            if (d == 3) r2 = r2 + f[2] * f[2];
                            pe_i += (double)u;
                            w_i += (double)(fr * r2);
                        }
                    }
                }
            }
        }
        out.potential += 0.5 * pe_i;
        out.virial += 0.5 * w_i;
    }
    return out;
}
// RDF pair counts over unordered pairs: bin k = floor(sqrt(r2) * (bins / rmax)) with r2 the f64
// square of the exact minimum-image separation.
inline std::vector<uint64_t> rdf_counts(const System& sys, const State& s, uint32_t bins, double rmax) {
    int d = sys.dim;
    std::vector<uint64_t> h(bins, 0);
    double scale = (double)bins / rmax;
    bool fits = true;
    {
        double bmax = 0.0;
        for (int a = 0; a < d; a++) bmax = std::max(bmax, sys.box_f64(a));
        for (int a = 0; a < d; a++)
            if (std::floor(sys.box_f64(a) / (rmax + 1e-3 + 1e-6 * bmax)) < 3.0) fits = false;
    }
    if (!fits) { // fewer than three cells of side rmax on an axis: every unordered pair once
        for (size_t i = 0; i < s.n(); i++)
            for (size_t j = i + 1; j < s.n(); j++) {
                double r2 = 0.0;
                for (int a = 0; a < d; a++) {
                    double dd = to_f64(sys.periodic(a) ? min_image(s.pos[d * i + a], s.pos[d * j + a], sys.box[a]) : s.pos[d * j + a] - s.pos[d * i + a]);
                    r2 = r2 + dd * dd;
                }
                double r = std::sqrt(r2) * scale;
                if (r < (double)bins) h[(uint32_t)r]++;
            }
        return h;
    }
    auto dims = sys.cells_for(rmax);
    CellList cl = build_cells(sys, s, dims);
    uint32_t nc[3] = {dims[0], dims[1], d == 3 ? dims[2] : 1u};
    for (size_t i = 0; i < s.n(); i++) {
        uint32_t key = cl.keys[i];
        uint32_t cc[3] = {key % nc[0], (key / nc[0]) % nc[1], key / (nc[0] * nc[1])};
        const int64_t* pi = &s.pos[d * i];
        std::vector<uint32_t> seen;
        int oz_n = d == 3 ? 3 : 1;
        for (int oz = 0; oz < oz_n; oz++) {
            uint32_t z = d == 3 ? (cc[2] + nc[2] + (uint32_t)oz - 1) % nc[2] : 0;
            for (int oy = 0; oy < 3; oy++) {
                uint32_t y = (cc[1] + nc[1] + (uint32_t)oy - 1) % nc[1];
                for (int ox = 0; ox < 3; ox++) {
                    uint32_t x = (cc[0] + nc[0] + (uint32_t)ox - 1) % nc[0];
                    uint32_t cell = (z * nc[1] + y) * nc[0] + x;
                    if (std::find(seen.begin(), seen.end(), cell) != seen.end()) continue;
                    seen.push_back(cell);
                    for (uint32_t q = cl.start[cell]; q < cl.start[cell + 1]; q++) {
                        uint32_t j = cl.items[q];
                        if (j <= i) continue;
                        double r2 = 0.0;
                        for (int a = 0; a < d; a++) {
                            double dd = to_f64(sys.periodic(a) ? min_image(pi[a], s.pos[d * j + a], sys.box[a]) : s.pos[d * j + a] - pi[a]);
                            r2 = r2 + dd * dd;
                        }
                        double r = std::sqrt(r2) * scale;
                        if (r < (double)bins) h[(uint32_t)r]++;
                    }
                }
            }
        }
    }
    return h;
}
// Particle counts in `bins` slabs along `axis`: bin = min(floor(x / L * bins), bins - 1) in f64.
inline std::vector<uint64_t> density_profile(const System& sys, const State& s, uint32_t bins, int axis) {
    std::vector<uint64_t> h(bins, 0);
    for (size_t i = 0; i < s.n(); i++) h[cell_of(to_f64(s.pos[sys.dim * i + axis]), sys.box_f64(axis), bins)]++;
    return h;
}
// Observer's density grid (crates/md/src/observe.rs:47-67, observe.wgsl:25-45): per particle the
// bin (min(u32(coord(x) sx), gx - 1), min(u32(coord(y) sy), gy - 1)) with coord(x) =
// f32(x_hi) + ldexp(f32(x_lo), -32) in f32 and s = (g / L) as f32; counts of all particles in
// out[0, gx gy), of species `marked` in out[gx gy, 2 gx gy).
inline uint32_t observer_bin(int64_t x, float scale, uint32_t g) {
    const uint64_t u = (uint64_t)x;
    const float c = (float)(uint32_t)(u >> 32) + std::ldexp((float)(uint32_t)u, -32);
    const float t = c * scale;
    const uint32_t b = (uint32_t)t; // t >= 0 and below 2^32 for a position in [0, L)
    return std::min(b, g - 1);
}
inline std::vector<uint32_t> observer_grid(const System& sys, const State& s, uint32_t gx, uint32_t gy, uint32_t marked) {
    std::vector<uint32_t> h(2 * (size_t)gx * gy, 0);
    const float sx = (float)((double)gx / sys.box_f64(0)), sy = (float)((double)gy / sys.box_f64(1));
    for (size_t i = 0; i < s.n(); i++) {
        const int64_t x = wrap(s.pos[2 * i], sys.box[0]), y = wrap(s.pos[2 * i + 1], sys.box[1]);
        const size_t b = (size_t)observer_bin(y, sy, gy) * gx + observer_bin(x, sx, gx);
        h[b]++;
        if (s.species[i] == marked) h[(size_t)gx * gy + b]++;
    }
    return h;
}
// The velocity-rescale thermostat of this engine: the half-step kinetic energy summed exactly as
// integers per species (sum of v^2 in 128 bits), then f = sqrt(t / now) as set_temperature
// (init.rs:92-103) with v <- round(v f) and an exact zero velocity sum.
inline double exact_half_step_kinetic(const System& sys, const State& s) {
    int d = sys.dim;
    unsigned __int128 acc[GBMD_MAX_SPECIES] = {0, 0, 0, 0};
    for (size_t i = 0; i < s.n(); i++) {
        uint32_t sp = s.species[i];
        if (sys.is_pinned(sp)) continue;
        for (int a = 0; a < d; a++) {
            int64_t v = s.vel[d * i + a];
            acc[sp] += (unsigned __int128)(uint64_t)(v * v);
        }
    }
    double ke = 0.0;
    double u = UNIT / sys.dt;
    for (int sp = 0; sp < sys.species(); sp++) {
        double hi = (double)(uint64_t)(acc[sp] >> 64) * 18446744073709551616.0;
        double sum = hi + (double)(uint64_t)acc[sp];
        ke += 0.5 * sys.masses[sp] * sum * (u * u);
    }
    return ke;
}
inline void rescale_temperature(State& s, const System& sys, double t) {
    int d = sys.dim;
    size_t moving = 0;
    for (size_t i = 0; i < s.n(); i++)
        if (!sys.is_pinned(s.species[i])) moving++;
    double dof = 0.5 * (double)d * std::max((double)moving - 1.0, 1.0);
    double now = exact_half_step_kinetic(sys, s) / dof;
    if (!(now > 0.0)) return;
    double f = std::sqrt(t / now);
    for (size_t i = 0; i < s.n(); i++) {
        if (sys.is_pinned(s.species[i])) continue;
        for (int a = 0; a < d; a++) s.vel[d * i + a] = sat_i32(std::round((double)s.vel[d * i + a] * f));
    }
    zero_velocity_sum(sys, s.species, s.vel, true);
}

} // namespace oracle
