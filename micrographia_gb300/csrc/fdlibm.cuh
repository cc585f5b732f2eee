// Sun's fdlibm 5.3 log, cos and sin (e_log.c, s_cos.c, s_sin.c, k_cos.c, k_sin.c,
// e_rem_pio2.c; the Rust crate `libm` 0.2.16 ports the same published algorithm) restated in IEEE
// double arithmetic on the device: every operation an explicit round-to-nearest intrinsic, in the
// published order, compiled without contraction. The seeded initial velocities (through the libm
// crate's Box-Muller) match the reference bit for bit with these; the Andersen bath's draws call
// Rust's f64::ln/cos/sin, the platform libm, which these match except where the two round a
// last bit differently.
#pragma once

#include <cstdint>

namespace gbmd {

static __device__ double dev_log(double x) {
    const double ln2_hi = 6.93147180369123816490e-01, ln2_lo = 1.90821492927058770002e-10;
    const double Lg1 = 6.666666666666735130e-01, Lg2 = 3.999999999940941908e-01, Lg3 = 2.857142874366239149e-01,
                 Lg4 = 2.222219843214978396e-01, Lg5 = 1.818357216161805012e-01, Lg6 = 1.531383769920937332e-01,
                 Lg7 = 1.479819860511658591e-01;
    uint64_t ui = (uint64_t)__double_as_longlong(x);
    uint32_t hx = (uint32_t)(ui >> 32);
    int k = 0;
    if (hx < 0x00100000u || (hx >> 31) != 0) {
        if ((ui << 1) == 0) return -1.0 / (x * x);
        if ((hx >> 31) != 0) return __longlong_as_double((long long)0xfff8000000000000ull); // log(x < 0): NaN (fdlibm's (x - x) / 0)
        k -= 54;
        x *= 18014398509481984.0;
        ui = (uint64_t)__double_as_longlong(x);
        hx = (uint32_t)(ui >> 32);
    } else if (hx >= 0x7ff00000u) {
        return x;
    } else if (hx == 0x3ff00000u && (ui << 32) == 0) {
        return 0.0;
    }
    hx += 0x3ff00000u - 0x3fe6a09eu;
    k += (int)(hx >> 20) - 0x3ff;
    hx = (hx & 0x000fffffu) + 0x3fe6a09eu;
    ui = ((uint64_t)hx << 32) | (ui & 0xffffffffull);
    x = __longlong_as_double((long long)ui);
    double f = __dsub_rn(x, 1.0);
    double hfsq = __dmul_rn(__dmul_rn(0.5, f), f);
    double s = __ddiv_rn(f, __dadd_rn(2.0, f));
    double z = __dmul_rn(s, s);
    double w = __dmul_rn(z, z);
    double t1 = __dmul_rn(w, __dadd_rn(Lg2, __dmul_rn(w, __dadd_rn(Lg4, __dmul_rn(w, Lg6)))));
    double t2 = __dmul_rn(z, __dadd_rn(Lg1, __dmul_rn(w, __dadd_rn(Lg3, __dmul_rn(w, __dadd_rn(Lg5, __dmul_rn(w, Lg7)))))));
    double r = __dadd_rn(t2, t1);
    double dk = (double)k;
    // s * (hfsq + r) + dk * ln2_lo - hfsq + f + dk * ln2_hi, left to right
    double acc = __dmul_rn(s, __dadd_rn(hfsq, r));
    acc = __dadd_rn(acc, __dmul_rn(dk, ln2_lo));
    acc = __dsub_rn(acc, hfsq);
    acc = __dadd_rn(acc, f);
    return __dadd_rn(acc, __dmul_rn(dk, ln2_hi));
}

static __device__ double dev_k_cos(double x, double y) {
    const double C1 = 4.16666666666666019037e-02, C2 = -1.38888888888741095749e-03, C3 = 2.48015872894767294178e-05,
                 C4 = -2.75573143513906633035e-07, C5 = 2.08757232129817482790e-09, C6 = -1.13596475577881948265e-11;
    double z = __dmul_rn(x, x);
    double w = __dmul_rn(z, z);
    double r = __dadd_rn(__dmul_rn(z, __dadd_rn(C1, __dmul_rn(z, __dadd_rn(C2, __dmul_rn(z, C3))))),
                         __dmul_rn(__dmul_rn(w, w), __dadd_rn(C4, __dmul_rn(z, __dadd_rn(C5, __dmul_rn(z, C6))))));
    double hz = __dmul_rn(0.5, z);
    w = __dsub_rn(1.0, hz);
    return __dadd_rn(w, __dadd_rn(__dsub_rn(__dsub_rn(1.0, w), hz), __dsub_rn(__dmul_rn(z, r), __dmul_rn(x, y))));
}

static __device__ double dev_k_sin(double x, double y, int iy) {
    const double S1 = -1.66666666666666324348e-01, S2 = 8.33333333332248946124e-03, S3 = -1.98412698298579493134e-04,
                 S4 = 2.75573137070700676789e-06, S5 = -2.50507602534068634195e-08, S6 = 1.58969099521155010221e-10;
    double z = __dmul_rn(x, x);
    double w = __dmul_rn(z, z);
    double r = __dadd_rn(__dadd_rn(S2, __dmul_rn(z, __dadd_rn(S3, __dmul_rn(z, S4)))),
                         __dmul_rn(__dmul_rn(z, w), __dadd_rn(S5, __dmul_rn(z, S6))));
    double v = __dmul_rn(z, x);
    if (iy == 0) return __dadd_rn(x, __dmul_rn(v, __dadd_rn(S1, __dmul_rn(z, r))));
    // x - ((z * (0.5 * y - v * r) - y) - v * S1)
    double inner = __dsub_rn(__dmul_rn(0.5, y), __dmul_rn(v, r));
    return __dsub_rn(x, __dsub_rn(__dsub_rn(__dmul_rn(z, inner), y), __dmul_rn(v, S1)));
}

static __device__ int dev_rem_pio2(double x, double& y0, double& y1) {
    const double toint = 1.5 / 2.220446049250313080847e-16, pio4 = 7.85398163397448278999e-01,
                 invpio2 = 6.36619772367581382433e-01, pio2_1 = 1.57079632673412561417e+00,
                 pio2_1t = 6.07710050650619224932e-11, pio2_2 = 6.07710050630396597660e-11,
                 pio2_2t = 2.02226624879595063154e-21, pio2_3 = 2.02226624871116645580e-21,
                 pio2_3t = 8.47842766036889956997e-32;
    uint64_t u = (uint64_t)__double_as_longlong(x);
    int sign = (int)(u >> 63);
    uint32_t ix = (uint32_t)(u >> 32) & 0x7fffffffu;
    bool medium = false;
    int quick = 0; // multiple of pi/2 for the quick paths
    if (ix <= 0x400f6a7au) {
        if ((ix & 0xfffffu) == 0x921fbu) medium = true;
        else quick = ix <= 0x4002d97cu ? 1 : 2;
    } else if (ix <= 0x401c463bu) {
        if (ix <= 0x4015fdbcu) {
            if (ix == 0x4012d97cu) medium = true;
            else quick = 3;
        } else {
            if (ix == 0x401921fbu) medium = true;
            else quick = 4;
        }
    } else {
        medium = true;
    }
    if (!medium) {
        double m = (double)quick;
        double p1 = __dmul_rn(m, pio2_1), p1t = __dmul_rn(m, pio2_1t);
        if (!sign) {
            double z = __dsub_rn(x, p1);
            y0 = __dsub_rn(z, p1t);
            y1 = __dsub_rn(__dsub_rn(z, y0), p1t);
            return quick;
        }
        double z = __dadd_rn(x, p1);
        y0 = __dadd_rn(z, p1t);
        y1 = __dadd_rn(__dsub_rn(z, y0), p1t);
        return -quick;
    }
    double fn = __dsub_rn(__dadd_rn(__dmul_rn(x, invpio2), toint), toint);
    int n = (int)fn;
    double r = __dsub_rn(x, __dmul_rn(fn, pio2_1));
    double w = __dmul_rn(fn, pio2_1t);
    if (__dsub_rn(r, w) < -pio4) {
        n--;
        fn = __dsub_rn(fn, 1.0);
        r = __dsub_rn(x, __dmul_rn(fn, pio2_1));
        w = __dmul_rn(fn, pio2_1t);
    } else if (__dsub_rn(r, w) > pio4) {
        n++;
        fn = __dadd_rn(fn, 1.0);
        r = __dsub_rn(x, __dmul_rn(fn, pio2_1));
        w = __dmul_rn(fn, pio2_1t);
    }
    y0 = __dsub_rn(r, w);
    int ey = (int)(((uint64_t)__double_as_longlong(y0) >> 52) & 0x7ff);
    int ex = (int)(ix >> 20);
    if (ex - ey > 16) {
        double t = r;
        w = __dmul_rn(fn, pio2_2);
        r = __dsub_rn(t, w);
        w = __dsub_rn(__dmul_rn(fn, pio2_2t), __dsub_rn(__dsub_rn(t, r), w));
        y0 = __dsub_rn(r, w);
        ey = (int)(((uint64_t)__double_as_longlong(y0) >> 52) & 0x7ff);
        if (ex - ey > 49) {
            t = r;
            w = __dmul_rn(fn, pio2_3);
            r = __dsub_rn(t, w);
            w = __dsub_rn(__dmul_rn(fn, pio2_3t), __dsub_rn(__dsub_rn(t, r), w));
            y0 = __dsub_rn(r, w);
        }
    }
    y1 = __dsub_rn(__dsub_rn(r, y0), w);
    return n;
}

static __device__ double dev_cos(double x) {
    uint32_t ix = (uint32_t)((uint64_t)__double_as_longlong(x) >> 32) & 0x7fffffffu;
    if (ix <= 0x3fe921fbu) {
        if (ix < 0x3e46a09eu && (int)x == 0) return 1.0;
        return dev_k_cos(x, 0.0);
    }
    if (ix >= 0x7ff00000u) return x - x;
    double y0, y1;
    int n = dev_rem_pio2(x, y0, y1);
    switch (n & 3) {
        case 0: return dev_k_cos(y0, y1);
        case 1: return -dev_k_sin(y0, y1, 1);
        case 2: return -dev_k_cos(y0, y1);
        default: return dev_k_sin(y0, y1, 1);
    }
}

static __device__ double dev_sin(double x) {
    uint32_t ix = (uint32_t)((uint64_t)__double_as_longlong(x) >> 32) & 0x7fffffffu;
    if (ix <= 0x3fe921fbu) {
        if (ix < 0x3e500000u) return x; // |x| < 2^-26
        return dev_k_sin(x, 0.0, 0);
    }
    if (ix >= 0x7ff00000u) return x - x;
    double y0, y1;
    int n = dev_rem_pio2(x, y0, y1);
    switch (n & 3) {
        case 0: return dev_k_sin(y0, y1, 1);
        case 1: return dev_k_cos(y0, y1);
        case 2: return -dev_k_sin(y0, y1, 1);
        default: return -dev_k_cos(y0, y1);
    }
}

} // namespace gbmd
