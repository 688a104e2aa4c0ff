// povgpu_quartic.cuh -- FP64 real-root solver for the torus quartic on the
// device.
//
// Same decision structure and tolerances as the reference's
// Solve_Polynomial (source/core/math/polynomialsolver.cpp:1585-1729) so
// that root sets agree: leading coefficients below 1e-10 are trimmed, a
// quartic whose constant term is negligible against the linear one
// (|c4/c3| < epsilon) drops to a cubic, coefficient spreads above 1e12
// switch from the closed form (Ferrari's resolvent cubic) to a Sturm
// sequence with bisection / regula falsi on [0, 1e7].  All loops are
// bounded (50 iterations per bracketing loop, 8 pending intervals).
#pragma once

namespace povgpu {
namespace quartic {

constexpr double SMALL_ENOUGH = 1.0e-10;
constexpr double RELERROR = 1.0e-12;
constexpr double FUDGE1 = 1.0e12;
constexpr double MAXD = 1.0e7;
constexpr int MAX_IT = 50;
constexpr double TWO_PI_3 = 2.0943951023931954923084;
constexpr double FOUR_PI_3 = 4.1887902047863909846168;

__device__ __forceinline__ int quadratic(const double* x, double* y)
{
    double a = x[0], b = -x[1], c = x[2];
    if (a == 0.0) {
        if (b == 0.0) return 0;
        y[0] = c / b;
        return 1;
    }
    b /= a;
    c /= a;
    double d = b * b - 4.0 * c;
    if (d > -SMALL_ENOUGH && d < SMALL_ENOUGH) {
        y[0] = 0.5 * b;
        return 1;
    }
    if (d < 0.0) return 0;
    d = sqrt(d);
    y[0] = (b + d) * 0.5;
    y[1] = (b - d) * 0.5;
    return 2;
}

// Cubic with the trigonometric form for three real roots and Cardano's
// form for one.
__device__ __forceinline__ int cubic(const double* x, double* y)
{
    double a0 = x[0];
    if (a0 == 0.0) return quadratic(x + 1, y);
    double a1, a2, a3;
    if (a0 != 1.0) { a1 = x[1] / a0; a2 = x[2] / a0; a3 = x[3] / a0; }
    else { a1 = x[1]; a2 = x[2]; a3 = x[3]; }
    double A2 = a1 * a1;
    double Q = (A2 - 3.0 * a2) / 9.0;
    double R = (a1 * (A2 - 4.5 * a2) + 13.5 * a3) / 27.0;
    double Q3 = Q * Q * Q, R2 = R * R, d = Q3 - R2, an = a1 / 3.0;
    if (d >= 0.0) {
        double th = acos(R / sqrt(Q3)) / 3.0;
        double sQ = -2.0 * sqrt(Q);
        y[0] = sQ * cos(th) - an;
        y[1] = sQ * cos(th + TWO_PI_3) - an;
        y[2] = sQ * cos(th + FOUR_PI_3) - an;
        return 3;
    }
    double sQ = pow(sqrt(R2 - Q3) + fabs(R), 1.0 / 3.0);
    y[0] = (R < 0 ? 1.0 : -1.0) * (sQ + Q / sQ) - an;
    return 1;
}

// Ferrari: depressed quartic, one root z of the resolvent cubic, two
// quadratic factors.
__device__ __forceinline__ int quartic_closed(const double* x, double* out)
{
    double c0 = x[0], c1, c2, c3, c4;
    if (c0 != 1.0) { c1 = x[1] / c0; c2 = x[2] / c0; c3 = x[3] / c0; c4 = x[4] / c0; }
    else { c1 = x[1]; c2 = x[2]; c3 = x[3]; c4 = x[4]; }
    double c12 = c1 * c1;
    double p = -0.375 * c12 + c2;
    double q = 0.125 * c12 * c1 - 0.5 * c1 * c2 + c3;
    double r = -0.01171875 * c12 * c12 + 0.0625 * c12 * c2 - 0.25 * c1 * c3 + c4;
    double cub[4] = {1.0, -0.5 * p, -r, 0.5 * r * p - 0.125 * q * q}, zr[3];
    if (cubic(cub, zr) <= 0) return 0;
    double z = zr[0];
    double d1 = 2.0 * z - p, d2;
    if (d1 < 0.0) {
        if (d1 > -SMALL_ENOUGH) d1 = 0.0;
        else return 0;
    }
    if (d1 < SMALL_ENOUGH) {
        d2 = z * z - r;
        if (d2 < 0.0) return 0;
        d2 = sqrt(d2);
    } else {
        d1 = sqrt(d1);
        d2 = 0.5 * q / d1;
    }
    double q1 = d1 * d1, q2 = -0.25 * c1;
    int n = 0;
    double e = q1 - 4.0 * (z - d2);
    if (e == 0) out[n++] = -0.5 * d1 - q2;
    else if (e > 0) {
        e = sqrt(e);
        out[n++] = -0.5 * (d1 + e) + q2;
        out[n++] = -0.5 * (d1 - e) + q2;
    }
    e = q1 - 4.0 * (z + d2);
    if (e == 0) out[n++] = 0.5 * d1 - q2;
    else if (e > 0) {
        e = sqrt(e);
        out[n++] = 0.5 * (d1 + e) + q2;
        out[n++] = 0.5 * (d1 - e) + q2;
    }
    return n;
}

// ----------------------------------------------------- Sturm sequence --
struct SPoly {
    int ord;
    double c[5];   // c[k] multiplies x^k
};

__device__ __forceinline__ double peval(double x, const SPoly& p)
{
    double v = p.c[p.ord];
    for (int i = p.ord - 1; i >= 0; i--)
        v = v * x + p.c[i];
    return v;
}

// remainder of u / v, sign-normalised as the Sturm recurrence wants
__device__ __forceinline__ int sturm_rem(const SPoly& u, const SPoly& v, SPoly& r)
{
    r = u;
    if (v.c[v.ord] < 0.0) {
        for (int k = u.ord - v.ord - 1; k >= 0; k -= 2)
            r.c[k] = -r.c[k];
        for (int k = u.ord - v.ord; k >= 0; k--)
            for (int j = v.ord + k - 1; j >= k; j--)
                r.c[j] = -r.c[j] - r.c[v.ord + k] * v.c[j - k];
    } else {
        for (int k = u.ord - v.ord; k >= 0; k--)
            for (int j = v.ord + k - 1; j >= k; j--)
                r.c[j] -= r.c[v.ord + k] * v.c[j - k];
    }
    int k = v.ord - 1;
    while (k >= 0 && fabs(r.c[k]) < SMALL_ENOUGH) {
        r.c[k] = 0.0;
        k--;
    }
    r.ord = k < 0 ? 0 : k;
    return r.ord;
}

__device__ __forceinline__ int sturm_build(int ord, SPoly* s)
{
    s[0].ord = ord;
    s[1].ord = ord - 1;
    double f = fabs(s[0].c[ord] * ord);
    for (int i = 1; i <= ord; i++)
        s[1].c[i - 1] = s[0].c[i] * i / f;
    int n = 2;
    while (n <= 4 && sturm_rem(s[n - 2], s[n - 1], s[n])) {
        double g = -fabs(s[n].c[s[n].ord]);
        for (int k = s[n].ord; k >= 0; k--)
            s[n].c[k] /= g;
        n++;
    }
    if (n > 4) n = 4;   // a quartic's sequence has at most 5 members
    s[n].c[0] = -s[n].c[0];
    return n;
}

__device__ __forceinline__ int sign_changes(int np, const SPoly* s, double a)
{
    int ch = 0;
    double lf = peval(a, s[0]);
    for (int i = 1; i <= np; i++) {
        double f = peval(a, s[i]);
        if (lf == 0.0 || lf * f < 0) ch++;
        lf = f;
    }
    return ch;
}

__device__ __forceinline__ bool falsi(const SPoly& p, double a, double b, double& val)
{
    double fa = peval(a, p), fb = peval(b, p), x = 0.0, fx, lfx;
    if (fa * fb > 0.0) return false;
    if (fabs(fa) < SMALL_ENOUGH) { val = a; return true; }
    if (fabs(fb) < SMALL_ENOUGH) { val = b; return true; }
    lfx = fa;
    for (int it = 0; it < MAX_IT; it++) {
        x = (fb * a - fa * b) / (fb - fa);
        fx = peval(x, p);
        if (fabs(x) > RELERROR ? fabs(fx / x) < RELERROR : fabs(fx) < RELERROR) { val = x; return true; }
        if ((fa < 0) == (fx < 0)) {
            a = x; fa = fx;
            if (lfx * fx > 0) fb /= 2;
        } else {
            b = x; fb = fx;
            if (lfx * fx > 0) fa /= 2;
        }
        if (fabs(b - a) < RELERROR) { val = x; return true; }
        lfx = fx;
    }
    return false;
}

__device__ __forceinline__ bool converged(double mn, double mx, double mid)
{
    return fabs(mid) > RELERROR ? fabs((mx - mn) / mid) < RELERROR : fabs(mx - mn) < RELERROR;
}

// Isolates the roots in [0, MAXD]: intervals holding several roots are
// bisected (pending intervals kept on a small explicit stack, left first),
// single-root intervals go to regula falsi, then bisection.
__device__ __forceinline__ int sturm_roots(int order, const double* cf, double* roots)
{
    SPoly s[5];
    for (int i = 0; i <= order; i++)
        s[0].c[order - i] = cf[i] / cf[0];
    int np = sturm_build(order, s);
    // visible roots: sign changes at 0 minus at +infinity
    int atinf = 0, atzero = 0;
    double lf = s[0].c[s[0].ord];
    for (int i = 1; i <= np; i++) {
        double f = s[i].c[s[i].ord];
        if (lf == 0.0 || lf * f < 0) atinf++;
        lf = f;
    }
    lf = s[0].c[0];
    for (int i = 1; i <= np; i++) {
        double f = s[i].c[0];
        if (lf == 0.0 || lf * f < 0) atzero++;
        lf = f;
    }
    if (atzero - atinf == 0) return 0;
    int amin = sign_changes(np, s, 0.0), amax = sign_changes(np, s, MAXD);
    if (amin - amax == 0) return 0;
    struct Iv { double lo, hi; int alo, ahi; };
    Iv st[8];
    int sp = 0, n = 0;
    st[sp++] = {0.0, MAXD, amin, amax};
    while (sp > 0 && n < 4) {
        Iv v = st[--sp];
        double mid = 0.5 * (v.lo + v.hi);
        if (v.alo - v.ahi == 1) {
            double r;
            if (falsi(s[0], v.lo, v.hi, r)) { roots[n++] = r; continue; }
            bool bad = false;
            for (int it = 0; it < MAX_IT; it++) {
                mid = 0.5 * (v.lo + v.hi);
                int am = sign_changes(np, s, mid);
                if (am < v.ahi || am > v.alo) { bad = true; break; }
                if (converged(v.lo, v.hi, mid)) break;
                if (v.alo - am == 0) v.lo = mid; else v.hi = mid;
            }
            if (!bad) roots[n++] = mid;
            continue;
        }
        bool split = false, bad = false;
        for (int it = 0; it < MAX_IT; it++) {
            mid = 0.5 * (v.lo + v.hi);
            int am = sign_changes(np, s, mid);
            if (am < v.ahi || am > v.alo) { bad = true; break; }
            if (converged(v.lo, v.hi, mid)) break;
            int n1 = v.alo - am, n2 = am - v.ahi;
            if (n1 != 0 && n2 != 0) {
                if (sp + 2 <= 8) {
                    st[sp++] = {mid, v.hi, am, v.ahi};   // right half handled after the left
                    st[sp++] = {v.lo, mid, v.alo, am};
                }
                split = true;
                break;
            }
            if (n1 == 0) v.lo = mid; else v.hi = mid;
        }
        if (!split && !bad) roots[n++] = mid;
    }
    return n;
}

__device__ __forceinline__ bool difficult(const double* x)
{
    double big = 0.0;
    for (int i = 0; i <= 4; i++)
        if (fabs(x[i]) > big) big = x[i];   // signed, as the reference keeps it
    if (big == 0.0) return false;
    for (int i = 0; i <= 4; i++)
        if (x[i] != 0.0 && fabs(big / x[i]) > FUDGE1) return true;
    return false;
}

// Solve_Polynomial(4, c, r, sturm = false, epsilon).
__device__ __forceinline__ int solve4(const double* c0, double* r, double epsilon)
{
    int i = 0;
    while (i < 4 && fabs(c0[i]) < SMALL_ENOUGH)
        i++;
    int n = 4 - i;
    const double* c = c0 + i;
    switch (n) {
    case 0: return 0;
    case 1:
        if (c[0] != 0.0) { r[0] = -c[1] / c[0]; return 1; }
        return 0;
    case 2: return quadratic(c, r);
    case 3:
        if (epsilon > 0.0 && c[2] != 0.0 && fabs(c[3] / c[2]) < epsilon) return quadratic(c, r);
        return cubic(c, r);
    default:
        if (epsilon > 0.0 && c[3] != 0.0 && fabs(c[4] / c[3]) < epsilon) return cubic(c, r);
        if (difficult(c)) return sturm_roots(4, c, r);
        return quartic_closed(c, r);
    }
}

}  // namespace quartic
}  // namespace povgpu
