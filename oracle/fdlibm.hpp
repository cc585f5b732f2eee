// ORACLE — test infrastructure only. Never linked into the engine.
//
// Restatement of the f64 `log` and `cos` that md-core's initial conditions call through the Rust
// crate `libm = 0.2.16` (Cargo.lock:406-407; call site crates/gpu-prims/src/threefry.rs:42-46).
// That crate is not vendored in the reference. Its `log` and `cos` are ports of the published
// FreeBSD msun / Sun fdlibm 5.3 algorithms (e_log.c; s_cos.c with k_cos.c, k_sin.c and the
// small-argument paths of e_rem_pio2.c), which this file restates: the same reduction, the same
// minimax polynomial coefficients and the same order of IEEE double operations, with no
// contraction into fused multiply-adds (build with -ffp-contract=off).
//
// Only the argument ranges the path uses matter here: log on (0, 1], cos on [0, 2 pi).
#pragma once

#include <cstdint>
#include <cstring>

namespace oracle {
namespace fdlibm {

inline uint64_t bits(double x) {
    uint64_t u;
    std::memcpy(&u, &x, 8);
    return u;
}
inline double from_bits(uint64_t u) {
    double x;
    std::memcpy(&x, &u, 8);
    return x;
}

// fdlibm e_log.c: log(x) = k ln2 + log(1 + f), f in [sqrt(2)/2 - 1, sqrt(2) - 1], with
// log(1 + f) = f - s (f - R(z)), s = f / (2 + f), R a degree-14 minimax polynomial in s.
inline double log(double x) {
    const double ln2_hi = 6.93147180369123816490e-01; /* 3fe62e42 fee00000 */
    const double ln2_lo = 1.90821492927058770002e-10; /* 3dea39ef 35793c76 */
    const double Lg1 = 6.666666666666735130e-01;      /* 3FE55555 55555593 */
    const double Lg2 = 3.999999999940941908e-01;      /* 3FD99999 9997FA04 */
    const double Lg3 = 2.857142874366239149e-01;      /* 3FD24924 94229359 */
    const double Lg4 = 2.222219843214978396e-01;      /* 3FCC71C5 1D8E78AF */
    const double Lg5 = 1.818357216161805012e-01;      /* 3FC74664 96CB03DE */
    const double Lg6 = 1.531383769920937332e-01;      /* 3FC39A09 D078C69F */
    const double Lg7 = 1.479819860511658591e-01;      /* 3FC2F112 DF3E5244 */

    uint64_t ui = bits(x);
    uint32_t hx = (uint32_t)(ui >> 32);
    int k = 0;
    if (hx < 0x00100000u || (hx >> 31) != 0) {
        if ((ui << 1) == 0) return -1.0 / (x * x); /* log(+-0) = -inf */
        if ((hx >> 31) != 0) return (x - x) / 0.0; /* log(-x) = NaN */
        /* subnormal: scale up by 2^54 */
        k -= 54;
        x *= 18014398509481984.0;
        ui = bits(x);
        hx = (uint32_t)(ui >> 32);
    } else if (hx >= 0x7ff00000u) {
        return x;
    } else if (hx == 0x3ff00000u && (ui << 32) == 0) {
        return 0.0;
    }
    /* reduce x into [sqrt(2)/2, sqrt(2)] */
    hx += 0x3ff00000u - 0x3fe6a09eu;
    k += (int)(hx >> 20) - 0x3ff;
    hx = (hx & 0x000fffffu) + 0x3fe6a09eu;
    ui = ((uint64_t)hx << 32) | (ui & 0xffffffffull);
    x = from_bits(ui);

    double f = x - 1.0;
    double hfsq = 0.5 * f * f;
    double s = f / (2.0 + f);
    double z = s * s;
    double w = z * z;
    double t1 = w * (Lg2 + w * (Lg4 + w * Lg6));
    double t2 = z * (Lg1 + w * (Lg3 + w * (Lg5 + w * Lg7)));
    double r = t2 + t1;
    double dk = (double)k;
    return s * (hfsq + r) + dk * ln2_lo - hfsq + f + dk * ln2_hi;
}

// fdlibm k_cos.c: cos(x + y) on [-pi/4, pi/4], y the tail of x.
inline double k_cos(double x, double y) {
    const double C1 = 4.16666666666666019037e-02;  /* 0x3FA55555, 0x5555554C */
    const double C2 = -1.38888888888741095749e-03; /* 0xBF56C16C, 0x16C15177 */
    const double C3 = 2.48015872894767294178e-05;  /* 0x3EFA01A0, 0x19CB1590 */
    const double C4 = -2.75573143513906633035e-07; /* 0xBE927E4F, 0x809C52AD */
    const double C5 = 2.08757232129817482790e-09;  /* 0x3E21EE9E, 0xBDB4B1C4 */
    const double C6 = -1.13596475577881948265e-11; /* 0xBDA8FAE9, 0xBE8838D4 */
    double z = x * x;
    double w = z * z;
    double r = z * (C1 + z * (C2 + z * C3)) + w * w * (C4 + z * (C5 + z * C6));
    double hz = 0.5 * z;
    w = 1.0 - hz;
    return w + (((1.0 - w) - hz) + (z * r - x * y));
}

// fdlibm k_sin.c: sin(x + y) on [-pi/4, pi/4]; iy = 0 if y is zero.
inline double k_sin(double x, double y, int iy) {
    const double S1 = -1.66666666666666324348e-01; /* 0xBFC55555, 0x55555549 */
    const double S2 = 8.33333333332248946124e-03;  /* 0x3F811111, 0x1110F8A6 */
    const double S3 = -1.98412698298579493134e-04; /* 0xBF2A01A0, 0x19C161D5 */
    const double S4 = 2.75573137070700676789e-06;  /* 0x3EC71DE3, 0x57B1FE7D */
    const double S5 = -2.50507602534068634195e-08; /* 0xBE5AE5E6, 0x8A2B9CEB */
    const double S6 = 1.58969099521155010221e-10;  /* 0x3DE5D93A, 0x5ACFD57C */
    double z = x * x;
    double w = z * z;
    double r = S2 + z * (S3 + z * S4) + z * w * (S5 + z * S6);
    double v = z * x;
    if (iy == 0) return x + v * (S1 + z * r);
    return x - ((z * (0.5 * y - v * r) - y) - v * S1);
}

// fdlibm e_rem_pio2.c for |x| < 2^20 pi/2: x = n pi/2 + (y0 + y1).
inline int rem_pio2(double x, double* y0, double* y1) {
    const double toint = 1.5 / 2.220446049250313080847e-16; /* 1.5 / DBL_EPSILON */
    const double pio4 = 7.85398163397448278999e-01;         /* 0x3FE921FB, 0x54442D18 */
    const double invpio2 = 6.36619772367581382433e-01;      /* 0x3FE45F30, 0x6DC9C883 */
    const double pio2_1 = 1.57079632673412561417e+00;       /* 0x3FF921FB, 0x54400000 */
    const double pio2_1t = 6.07710050650619224932e-11;      /* 0x3DD0B461, 0x1A626331 */
    const double pio2_2 = 6.07710050630396597660e-11;       /* 0x3DD0B461, 0x1A600000 */
    const double pio2_2t = 2.02226624879595063154e-21;      /* 0x3BA3198A, 0x2E037073 */
    const double pio2_3 = 2.02226624871116645580e-21;       /* 0x3BA3198A, 0x2E000000 */
    const double pio2_3t = 8.47842766036889956997e-32;      /* 0x397B839A, 0x252049C1 */

    uint64_t u = bits(x);
    int sign = (int)(u >> 63);
    uint32_t ix = (uint32_t)(u >> 32) & 0x7fffffffu;
    bool medium = false;
    if (ix <= 0x400f6a7au) { /* |x| ~<= 5pi/4 */
        if ((ix & 0xfffffu) == 0x921fbu) {
            medium = true; /* |x| ~= pi/2 or 2pi/2: cancellation */
        } else if (ix <= 0x4002d97cu) { /* |x| ~<= 3pi/4 */
            if (!sign) {
                double z = x - pio2_1;
                *y0 = z - pio2_1t;
                *y1 = (z - *y0) - pio2_1t;
                return 1;
            } else {
                double z = x + pio2_1;
                *y0 = z + pio2_1t;
                *y1 = (z - *y0) + pio2_1t;
                return -1;
            }
        } else {
            if (!sign) {
                double z = x - 2.0 * pio2_1;
                *y0 = z - 2.0 * pio2_1t;
                *y1 = (z - *y0) - 2.0 * pio2_1t;
                return 2;
            } else {
                double z = x + 2.0 * pio2_1;
                *y0 = z + 2.0 * pio2_1t;
                *y1 = (z - *y0) + 2.0 * pio2_1t;
                return -2;
            }
        }
    }
    if (!medium && ix <= 0x401c463bu) { /* |x| ~<= 9pi/4 */
        if (ix <= 0x4015fdbcu) {        /* |x| ~<= 7pi/4 */
            if (ix == 0x4012d97cu) {
                medium = true; /* |x| ~= 3pi/2 */
            } else if (!sign) {
                double z = x - 3.0 * pio2_1;
                *y0 = z - 3.0 * pio2_1t;
                *y1 = (z - *y0) - 3.0 * pio2_1t;
                return 3;
            } else {
                double z = x + 3.0 * pio2_1;
                *y0 = z + 3.0 * pio2_1t;
                *y1 = (z - *y0) + 3.0 * pio2_1t;
                return -3;
            }
        } else {
            if (ix == 0x401921fbu) {
                medium = true; /* |x| ~= 4pi/2 */
            } else if (!sign) {
                double z = x - 4.0 * pio2_1;
                *y0 = z - 4.0 * pio2_1t;
                *y1 = (z - *y0) - 4.0 * pio2_1t;
                return 4;
            } else {
                double z = x + 4.0 * pio2_1;
                *y0 = z + 4.0 * pio2_1t;
                *y1 = (z - *y0) + 4.0 * pio2_1t;
                return -4;
            }
        }
    }
    /* medium size: |x| < 2^20 pi/2 (the only other case the path reaches) */
    double fn = x * invpio2 + toint - toint;
    int n = (int)fn;
    double r = x - fn * pio2_1;
    double w = fn * pio2_1t;
    if (r - w < -pio4) {
        n--;
        fn--;
        r = x - fn * pio2_1;
        w = fn * pio2_1t;
    } else if (r - w > pio4) {
        n++;
        fn++;
        r = x - fn * pio2_1;
        w = fn * pio2_1t;
    }
    *y0 = r - w;
    int ey = (int)((bits(*y0) >> 52) & 0x7ff);
    int ex = (int)(ix >> 20);
    if (ex - ey > 16) { /* second round, good to 118 bits */
        double t = r;
        w = fn * pio2_2;
        r = t - w;
        w = fn * pio2_2t - ((t - r) - w);
        *y0 = r - w;
        ey = (int)((bits(*y0) >> 52) & 0x7ff);
        if (ex - ey > 49) { /* third round, good to 151 bits */
            t = r;
            w = fn * pio2_3;
            r = t - w;
            w = fn * pio2_3t - ((t - r) - w);
            *y0 = r - w;
        }
    }
    *y1 = (r - *y0) - w;
    return n;
}

// fdlibm s_cos.c.
inline double cos(double x) {
    uint32_t ix = (uint32_t)(bits(x) >> 32) & 0x7fffffffu;
    if (ix <= 0x3fe921fbu) {      /* |x| ~< pi/4 */
        if (ix < 0x3e46a09eu) {   /* |x| < 2^-27 sqrt(2) */
            if ((int)x == 0) return 1.0;
        }
        return k_cos(x, 0.0);
    }
    if (ix >= 0x7ff00000u) return x - x;
    double y0, y1;
    int n = rem_pio2(x, &y0, &y1);
    switch (n & 3) {
        case 0: return k_cos(y0, y1);
        case 1: return -k_sin(y0, y1, 1);
        case 2: return -k_cos(y0, y1);
        default: return k_sin(y0, y1, 1);
    }
}

// s_sin.c: the same reduction, the kernels rotated by a quarter turn.
inline double sin(double x) {
    uint32_t ix = (uint32_t)(bits(x) >> 32) & 0x7fffffffu;
    if (ix <= 0x3fe921fbu) {    /* |x| ~< pi/4 */
        if (ix < 0x3e500000u) { /* |x| < 2^-26 */
            if ((int)x == 0) return x;
        }
        return k_sin(x, 0.0, 0);
    }
    if (ix >= 0x7ff00000u) return x - x;
    double y0, y1;
    int n = rem_pio2(x, &y0, &y1);
    switch (n & 3) {
        case 0: return k_sin(y0, y1, 1);
        case 1: return k_cos(y0, y1);
        case 2: return -k_sin(y0, y1, 1);
        default: return -k_cos(y0, y1);
    }
}

} // namespace fdlibm
} // namespace oracle
