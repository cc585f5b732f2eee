// Seeded initial conditions generated on the device: md-core's init::lattice / init::maxwell /
// init::zero_velocity_sum (crates/md-core/src/init.rs:22-89), three::fcc / three::maxwell /
// three::zero_velocity_sum (crates/md-core/src/three.rs:319-389), and this engine's triangular
// lattice and liquid-vapour slab. Bit-identical to the CPU definitions: the same Threefry
// counters, the same f64 operation order (no contraction: -fmad=false), and the same libm.
//
// The Maxwell draws call libm's log and cos through gpu-prims' Box–Muller
// (crates/gpu-prims/src/threefry.rs:42-46), i.e. the Rust crate `libm = 0.2.16` (Cargo.lock:
// 406-407), whose log and cos are ports of Sun's fdlibm 5.3 (e_log.c, s_cos.c, k_cos.c,
// k_sin.c, e_rem_pio2.c). dev_log / dev_cos (fdlibm.cuh) restate that published algorithm in IEEE
// double arithmetic, so the velocities match the reference's bit for bit; CUDA's own log/cos
// would differ in the last ulp now and then, and a rounded velocity with them.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "engine.cuh"
#include "fdlibm.cuh"
#include "sort.cuh"

namespace gbmd {

namespace {

// threefry::normal (threefry.rs:42-46): Box–Muller on uniforms 2i and 2i + 1.
__device__ double dev_normal(uint64_t seed, uint32_t stream, uint32_t i) {
    double u1 = __dsub_rn(1.0, uniform01(seed, stream, 2u * i));
    double u2 = uniform01(seed, stream, 2u * i + 1u);
    return __dmul_rn(__dsqrt_rn(__dmul_rn(-2.0, dev_log(u1))), dev_cos(__dmul_rn(6.28318530717958647692, u2)));
}

constexpr uint32_t STREAM_VELOCITY = 1, STREAM_JITTER = 2, STREAM_DIRECTION = 3, STREAM_VAPOUR = 4;

// ---------------------------------------------------------------- position kernels
struct Lattice2 {
    uint32_t nx;
    double a0, a1;
    int64_t origin[2];
    int64_t wrap_len[2];
    int64_t post[2]; // added after the wrap (init::fluid's 1 sigma clear of a wall)
    double jitter;
    uint64_t seed;
    uint32_t first_id; // id of site 0 (jitter counters and the output slot)
    uint32_t count;
    int triangular;
};

// init::lattice (init.rs:22-38) and the triangular variant (oracle triangular()).
__global__ void k_lattice2(Lattice2 L, longlong2* pos) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L.count) return;
    uint32_t i = k % L.nx, j = k / L.nx;
    uint32_t id = L.first_id + k;
    double jx = __dmul_rn(L.jitter, __dsub_rn(uniform01(L.seed, STREAM_JITTER, 2u * id), 0.5));
    double jy = __dmul_rn(L.jitter, __dsub_rn(uniform01(L.seed, STREAM_JITTER, 2u * id + 1u), 0.5));
    double cx = L.triangular ? __dadd_rn((double)i, (j & 1) ? 0.75 : 0.25) : __dadd_rn((double)i, 0.5);
    double cy = __dadd_rn((double)j, 0.5);
    int64_t x = L.origin[0] + to_fixed(__dadd_rn(__dmul_rn(cx, L.a0), jx));
    int64_t y = L.origin[1] + to_fixed(__dadd_rn(__dmul_rn(cy, L.a1), jy));
    pos[id] = make_longlong2(wrap(x, L.wrap_len[0]) + L.post[0], wrap(y, L.wrap_len[1]) + L.post[1]);
}

struct Vapour2 {
    uint32_t vx, first_id, count;
    double ax, ay, room_x, room_y;
    int64_t x1, lx, ly;
    uint64_t seed;
};
// The slab's vapour: a square lattice with per-site uniform displacements (oracle slab()).
__global__ void k_vapour2(Vapour2 V, longlong2* pos) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= V.count) return;
    uint32_t i = k % V.vx, j = k / V.vx;
    double ux = uniform01(V.seed, STREAM_VAPOUR, 2u * k), uy = uniform01(V.seed, STREAM_VAPOUR, 2u * k + 1u);
    double x = __dadd_rn(__dadd_rn(__dmul_rn((double)i, V.ax), __dmul_rn(0.5, __dsub_rn(V.ax, V.room_x))), __dmul_rn(ux, V.room_x));
    double y = __dadd_rn(__dadd_rn(__dmul_rn((double)j, V.ay), __dmul_rn(0.5, __dsub_rn(V.ay, V.room_y))), __dmul_rn(uy, V.room_y));
    int64_t xf = wrap(V.x1 + to_fixed(__dadd_rn(1.0, x)), V.lx);
    pos[V.first_id + k] = make_longlong2(xf, wrap(to_fixed(y), V.ly));
}

struct Fcc3 {
    uint32_t n, cx, cy;
    double a[3];
    int64_t box[3];
    double jitter;
    uint64_t seed;
};
// three::fcc (three.rs:319-343): sites in (z, y, x, basis) order.
__global__ void k_fcc3(Fcc3 F, longlong4_32a* pos) {
    uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= F.n) return;
    const double basis[4][3] = {{0.25, 0.25, 0.25}, {0.75, 0.75, 0.25}, {0.75, 0.25, 0.75}, {0.25, 0.75, 0.75}};
    uint32_t s = id & 3u, cell = id >> 2;
    uint32_t c[3] = {cell % F.cx, (cell / F.cx) % F.cy, cell / (F.cx * F.cy)};
    int64_t x[3];
    for (int ax = 0; ax < 3; ax++) {
        double jit = __dmul_rn(F.jitter, __dsub_rn(uniform01(F.seed, STREAM_JITTER, 3u * id + (uint32_t)ax), 0.5));
        x[ax] = wrap(to_fixed(__dadd_rn(__dmul_rn(__dadd_rn((double)c[ax], basis[s][ax]), F.a[ax]), jit)), F.box[ax]);
    }
    longlong2* q = reinterpret_cast<longlong2*>(pos + id);
    q[0] = make_longlong2(x[0], x[1]);
    q[1] = make_longlong2(x[2], 0);
}

// ---------------------------------------------------------------- Maxwell velocities
struct MaxwellP {
    uint32_t n, dim;
    double t, dt;
    double masses[GBMD_MAX_SPECIES];
    uint32_t pinned;
    uint64_t seed;
};
// init::maxwell (init.rs:42-57) / three::maxwell (three.rs:359-373): draw d i + a.
__global__ void k_maxwell(MaxwellP M, const uint32_t* species, int32_t* vel) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M.n) return;
    uint32_t s = species[i];
    bool skip = M.dim == 3 && ((M.pinned >> s) & 1u);
    double sd = __dsqrt_rn(__ddiv_rn(M.t, M.masses[s]));
    for (uint32_t a = 0; a < M.dim; a++) {
        int32_t v = 0;
        if (!skip) {
            double x = __dmul_rn(sd, dev_normal(M.seed, STREAM_VELOCITY, M.dim * i + a));
            // System::to_step_displacement (system.rs:427-429): round(v dt 2^32) as i32
            v = sat_i32_f64(round(__dmul_rn(__dmul_rn(x, M.dt), 4294967296.0)));
        }
        vel[M.dim * i + a] = v;
    }
}

// init::fixed_speed (init.rs:61-74), 2D: every particle at speed sqrt(2 t / m) in the direction
// TAU u, u = uniform(seed, STREAM_DIRECTION, i), cos and sin as fdlibm's.
__global__ void k_fixed_speed(MaxwellP M, const uint32_t* species, int32_t* vel) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M.n) return;
    const double speed = __dsqrt_rn(__ddiv_rn(__dmul_rn(2.0, M.t), M.masses[species[i]]));
    const double th = __dmul_rn(6.28318530717958647692, uniform01(M.seed, STREAM_DIRECTION, i));
    vel[2 * i] = sat_i32_f64(round(__dmul_rn(__dmul_rn(__dmul_rn(speed, dev_cos(th)), M.dt), 4294967296.0)));
    vel[2 * i + 1] = sat_i32_f64(round(__dmul_rn(__dmul_rn(__dmul_rn(speed, dev_sin(th)), M.dt), 4294967296.0)));
}

__global__ void k_moving_flags(const uint32_t* species, uint32_t n, uint32_t pinned, int skip_pinned, uint32_t* flags) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flags[i] = (skip_pinned && ((pinned >> species[i]) & 1u)) ? 0u : 1u;
}

// Per-block sums of the velocity components of moving particles (exact, i64).
__global__ void k_vel_sums(const int32_t* vel, const uint32_t* flags, uint32_t n, uint32_t dim, long long* partial) {
    __shared__ long long sh[3][32];
    long long acc[3] = {0, 0, 0};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (flags[i])
            for (uint32_t a = 0; a < dim; a++) acc[a] += vel[dim * i + a];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int a = 0; a < 3; a++) {
        long long v = acc[a];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[a][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        long long s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += sh[threadIdx.x][w];
        partial[blockIdx.x * 3 + threadIdx.x] = s;
    }
}

// The per-block sums added up in order: totals[a] (in place at partial[3 * nblocks + a]).
__global__ void k_sum_partials(long long* partial, uint32_t nblocks) {
    for (int a = 0; a < 3; a++) {
        long long s = 0;
        for (uint32_t b = 0; b < nblocks; b++) s += partial[b * 3 + a];
        partial[3 * nblocks + a] = s;
    }
}

// zero_velocity_sum: q = div_euclid(sum, m), r = rem_euclid(sum, m); the k-th moving particle
// (in id order) loses q + (k < r). rank[i] is i's index among moving particles.
__global__ void k_zero_sum(int32_t* vel, const uint32_t* flags, const uint32_t* rank, uint32_t n, uint32_t dim, const long long* totals,
                           uint32_t moving) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !flags[i] || moving == 0) return;
    long long m = moving;
    for (uint32_t a = 0; a < dim; a++) {
        long long sum = totals[a];
        long long q = sum / m, r = sum % m;
        if (r < 0) {
            q -= 1;
            r += m;
        }
        long long sub = q + ((long long)rank[i] < r ? 1 : 0);
        vel[dim * i + a] = (int32_t)((uint32_t)vel[dim * i + a] - (uint32_t)sub);
    }
}

uint32_t blocks(uint64_t n, uint32_t t) { return (uint32_t)((n + t - 1) / t); }

double host_to_f64(int64_t x) { return (double)x * (1.0 / 4294967296.0); }
int64_t host_to_fixed(double x) {
    double r = std::round(x * 4294967296.0);
    if (r != r) return 0;
    if (r >= 9223372036854775807.0) return INT64_MAX;
    if (r <= -9223372036854775808.0) return INT64_MIN;
    return (int64_t)r;
}
uint32_t host_sat_u32(double x) {
    if (!(x > 0.0)) return 0;
    if (x >= 4294967295.0) return UINT32_MAX;
    return (uint32_t)x;
}

} // namespace

// ---------------------------------------------------------------- host-side shapes
// init::lattice's nx (init.rs:24-25)
static uint32_t lattice_nx(uint64_t n, double b0, double b1) {
    return std::max<uint32_t>(host_sat_u32(std::ceil(std::sqrt((double)n * b0 / b1))), 1);
}
// The triangular lattice's shape: nx = round(sqrt(n (Lx / Ly) sqrt(3)/2)), ny even.
static void triangular_shape(uint64_t n, double b0, double b1, uint32_t* nx, uint32_t* ny) {
    uint32_t x = std::max<uint32_t>(host_sat_u32(std::round(std::sqrt((double)n * (b0 / b1) * 0.86602540378443864676))), 1);
    uint64_t y = (n + x - 1) / x;
    if (y > 1 && (y & 1)) y++;
    *nx = x;
    *ny = (uint32_t)y;
}
// three::fcc_cells (three.rs:346-355)
static void fcc_cells(uint64_t n, const int64_t* box, uint64_t* c) {
    double b[3] = {host_to_f64(box[0]), host_to_f64(box[1]), host_to_f64(box[2])};
    double a = std::cbrt(b[0] * b[1] * b[2] * 4.0 / (double)n);
    for (int k = 0; k < 3; k++) c[k] = std::max<uint64_t>(host_sat_u32(std::round(b[k] / a)), 1);
    while (4 * c[0] * c[1] * c[2] < n) {
        int k = 0;
        for (int x = 1; x < 3; x++)
            if (b[x] / (double)c[x] > b[k] / (double)c[k]) k = x;
        c[k]++;
    }
}

static int launch_lattice(const Lattice2& L, longlong2* pos, cudaStream_t s) {
    if (L.count) k_lattice2<<<blocks(L.count, 256), 256, 0, s>>>(L, pos);
    note_launch();
    return GBMD_OK;
}

// Velocities: Maxwell draws, then the exact zero sum over moving particles in id order.
static int maxwell_device(const gbmd_system& sys, uint32_t n, double t, uint64_t seed, const uint32_t* species, int32_t* vel,
                          cudaStream_t s, bool fixed_speed = false) {
    if (n == 0) return GBMD_OK;
    MaxwellP M;
    M.n = n;
    M.dim = sys.dim;
    M.t = t;
    M.dt = sys.dt;
    for (int k = 0; k < GBMD_MAX_SPECIES; k++) M.masses[k] = k < (int)sys.nspecies ? sys.masses[k] : 1.0;
    M.pinned = sys.pinned;
    M.seed = seed;
    if (fixed_speed) k_fixed_speed<<<blocks(n, 128), 128, 0, s>>>(M, species, vel);
    else k_maxwell<<<blocks(n, 128), 128, 0, s>>>(M, species, vel);
    note_launch();
    const uint32_t nb = std::min<uint32_t>(blocks(n, 256), 1024);
    uint32_t *flags = nullptr, *rank = nullptr, *tmp = nullptr;
    long long* partial = nullptr;
    size_t tmp_n = scan_tmp_elems(n);
    GBMD_CUDA_TRY(cudaMallocAsync(&flags, (size_t)n * 4, s));
    GBMD_CUDA_TRY(cudaMallocAsync(&rank, (size_t)n * 4, s));
    GBMD_CUDA_TRY(cudaMallocAsync(&tmp, tmp_n * 4, s));
    GBMD_CUDA_TRY(cudaMallocAsync(&partial, ((size_t)nb + 1) * 3 * 8, s));
    int skip = sys.dim == 3;
    k_moving_flags<<<blocks(n, 256), 256, 0, s>>>(species, n, sys.pinned, skip, flags);
    scan_exclusive(flags, rank, n, tmp, s);
    k_vel_sums<<<nb, 256, 0, s>>>(vel, flags, n, sys.dim, partial);
    k_sum_partials<<<1, 1, 0, s>>>(partial, nb);
    // the number of moving particles: rank of the last + its flag
    uint32_t last_rank = 0, last_flag = 0;
    GBMD_CUDA_TRY(cudaMemcpyAsync(&last_rank, rank + n - 1, 4, cudaMemcpyDeviceToHost, s));
    GBMD_CUDA_TRY(cudaMemcpyAsync(&last_flag, flags + n - 1, 4, cudaMemcpyDeviceToHost, s));
    GBMD_CUDA_TRY(cudaStreamSynchronize(s));
    k_zero_sum<<<blocks(n, 256), 256, 0, s>>>(vel, flags, rank, n, sys.dim, partial + 3 * (size_t)nb, last_rank + last_flag);
    note_launch(6);
    cudaFreeAsync(flags, s);
    cudaFreeAsync(rank, s);
    cudaFreeAsync(tmp, s);
    cudaFreeAsync(partial, s);
    GBMD_CUDA_TRY(cudaGetLastError());
    return GBMD_OK;
}

int maxwell_state_device(const gbmd_system& sys, uint32_t n, double t, uint64_t seed, const uint32_t* species_dev, int32_t* vel_dev,
                         cudaStream_t s, bool fixed_speed) {
    if (fixed_speed && sys.dim != 2) return fail(GBMD_E_UNSUPPORTED, "fixed_speed is two-dimensional (init::fixed_speed)");
    return maxwell_device(sys, n, t, seed, species_dev, vel_dev, s, fixed_speed);
}

int init_state_device(const gbmd_system& sys, const gbmd_init& spec, void* pos_dev, int32_t* vel_dev, uint32_t* species_dev, cudaStream_t s) {
    uint32_t n = spec.n;
    if (n == 0) return GBMD_OK;
    GBMD_CUDA_TRY(cudaMemsetAsync(species_dev, 0, (size_t)n * 4, s));
    double b0 = host_to_f64(sys.box_len[0]), b1 = host_to_f64(sys.box_len[1]);
    switch (spec.recipe) {
        case GBMD_INIT_FLUID:
        case GBMD_INIT_TRIANGULAR: {
            if (sys.dim != 2) return fail(GBMD_E_INVALID, "2D recipe on a 3D system");
            Lattice2 L{};
            uint32_t nx, ny;
            // init::fluid (init.rs:105-121): on an axis with walls the lattice fills the box less
            // 2 sigma and is then moved 1 sigma in, clear of the walls
            int64_t inner[2] = {sys.box_len[0], sys.box_len[1]};
            if (spec.recipe == GBMD_INIT_FLUID) {
                for (int a = 0; a < 2; a++)
                    if (!((sys.periodic >> a) & 1u)) {
                        inner[a] = sys.box_len[a] - host_to_fixed(2.0);
                        L.post[a] = host_to_fixed(1.0);
                    }
                if (inner[0] <= 0 || inner[1] <= 0) return fail(GBMD_E_INVALID, "a walled axis is too short for the fluid lattice");
                b0 = host_to_f64(inner[0]);
                b1 = host_to_f64(inner[1]);
                nx = lattice_nx(n, b0, b1);
                ny = (uint32_t)(((uint64_t)n + nx - 1) / nx);
            } else {
                if ((sys.periodic & 3u) != 3u) return fail(GBMD_E_UNSUPPORTED, "the triangular recipe is for periodic boxes");
                triangular_shape(n, b0, b1, &nx, &ny);
            }
            L.nx = nx;
            L.a0 = b0 / (double)nx;
            L.a1 = b1 / (double)ny;
            L.wrap_len[0] = inner[0];
            L.wrap_len[1] = inner[1];
            L.jitter = spec.jitter;
            L.seed = spec.seed;
            L.count = n;
            L.triangular = spec.recipe == GBMD_INIT_TRIANGULAR;
            GBMD_TRY(launch_lattice(L, (longlong2*)pos_dev, s));
            break;
        }
        case GBMD_INIT_SLAB: {
            if (sys.dim != 2) return fail(GBMD_E_INVALID, "the slab recipe is 2D");
            if ((sys.periodic & 3u) != 3u) return fail(GBMD_E_UNSUPPORTED, "the slab recipe is for periodic boxes");
            double lx = b0, ly = b1, frac = spec.slab_frac;
            int64_t x0 = host_to_fixed(lx * (1.0 - frac) * 0.5), x1 = host_to_fixed(lx * (1.0 + frac) * 0.5);
            double wl = host_to_f64(x1 - x0);
            uint32_t n_l = std::min<uint32_t>(n, host_sat_u32(std::round(spec.rho_liquid * wl * ly)));
            uint32_t n_v = n - n_l;
            double wv = std::max(lx - wl - 2.0, 0.0);
            uint32_t vy = std::max<uint32_t>(host_sat_u32(std::ceil(std::sqrt((double)n_v * ly / std::max(wv, 1e-9)))), 1);
            uint32_t vx = n_v ? (n_v + vy - 1) / vy : 0;
            Lattice2 L{};
            uint32_t nx, ny;
            triangular_shape(n_l, wl, ly, &nx, &ny);
            L.nx = nx;
            L.a0 = wl / (double)nx;
            L.a1 = ly / (double)ny;
            L.origin[0] = x0;
            L.wrap_len[0] = sys.box_len[0];
            L.wrap_len[1] = sys.box_len[1];
            L.jitter = spec.jitter;
            L.seed = spec.seed;
            L.count = n_l;
            L.triangular = 1;
            GBMD_TRY(launch_lattice(L, (longlong2*)pos_dev, s));
            if (n_v) {
                Vapour2 V{};
                V.vx = vx;
                V.first_id = n_l;
                V.count = n_v;
                V.ax = wv / (double)vx;
                V.ay = ly / (double)vy;
                V.room_x = std::max(V.ax - 1.0, 0.0);
                V.room_y = std::max(V.ay - 1.0, 0.0);
                V.x1 = x1;
                V.lx = sys.box_len[0];
                V.ly = sys.box_len[1];
                V.seed = spec.seed;
                k_vapour2<<<blocks(n_v, 256), 256, 0, s>>>(V, (longlong2*)pos_dev);
                note_launch();
            }
            break;
        }
        case GBMD_INIT_FCC: {
            if (sys.dim != 3) return fail(GBMD_E_INVALID, "the FCC recipe is 3D");
            uint64_t c[3];
            fcc_cells(n, sys.box_len, c);
            Fcc3 F{};
            F.n = n;
            F.cx = (uint32_t)c[0];
            F.cy = (uint32_t)c[1];
            for (int a = 0; a < 3; a++) {
                F.a[a] = host_to_f64(sys.box_len[a]) / (double)c[a];
                F.box[a] = sys.box_len[a];
            }
            F.jitter = spec.jitter;
            F.seed = spec.seed;
            k_fcc3<<<blocks(n, 256), 256, 0, s>>>(F, (longlong4_32a*)pos_dev);
            note_launch();
            break;
        }
        default:
            return fail(GBMD_E_INVALID, "unknown init recipe");
    }
    GBMD_TRY(maxwell_device(sys, n, spec.t, spec.seed, species_dev, vel_dev, s));
    GBMD_CUDA_TRY(cudaGetLastError());
    return GBMD_OK;
}

} // namespace gbmd
