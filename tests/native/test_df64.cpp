// Host unit test of the float-float arithmetic (lgpu_df64.cuh) used by the
// complex128 fused gate bodies:
//  * df_from_double keeps d within 2^-47 |d| + 2^-126 (|d| < 2^-126 -> 0);
//  * df_to_double is exact for normalised pairs and within one double ulp
//    otherwise;
//  * every structured body agrees with a long-double evaluation of the same
//    2x2 product within 4e-14 of the largest input magnitude;
//  * NaN inputs give NaN outputs;
//  * df_expval_group (3-target expectations) agrees with long double.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>

#include "lgpu_df64.cuh"

using lgpu::DF;

static long bad = 0;

static void fail(const char *what, double a, double b) {
    if (bad < 20) std::printf("bad %s: %a vs %a\n", what, a, b);
    bad++;
}

int main() {
    std::mt19937_64 gen(7);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    std::uniform_int_distribution<int> ex(-120, 4);
    long n_split = 0, n_rebuild = 0, n_body = 0;

    // split
    for (int i = 0; i < 2000000; i++) {
        const double d = std::ldexp(u(gen), ex(gen));
        const DF r = lgpu::df_from_double(d);
        const double back = double(r.hi) + double(r.lo);
        n_split++;
        if (std::fabs(d) < std::ldexp(1.0, -126)) {
            if (back != 0.0) fail("split tiny", d, back);
        } else if (std::fabs(back - d) > std::ldexp(std::fabs(d), -47) + std::ldexp(1.0, -126)) {
            fail("split", d, back);
        }
    }
    for (double d : {0.0, -0.0, 1.0, -1.0, 0.5, 1e-300, 3e-310, 1e-38, 2e-38, 0.7071067811865476, 1e30}) {
        const DF r = lgpu::df_from_double(d);
        const double back = double(r.hi) + double(r.lo);
        if (std::fabs(back - d) > std::ldexp(std::fabs(d), -47) + std::ldexp(1.0, -126)) fail("split edge", d, back);
    }

    // rebuild: normalised pairs are exact; loose pairs within one ulp
    for (int i = 0; i < 2000000; i++) {
        const double d = std::ldexp(u(gen), ex(gen) / 2);
        const DF r = lgpu::df_split_host(d);
        const double ref = double(r.hi) + double(r.lo);
        const double got = lgpu::df_to_double(r);
        n_rebuild++;
        if (got != ref) fail("rebuild normalised", ref, got);
        DF loose{float(u(gen)), float(std::ldexp(u(gen), -(i % 40)))};
        const double lref = double(loose.hi) + double(loose.lo);
        const double lgot = lgpu::df_to_double(loose);
        const double ulp = std::fabs(std::nextafter(lref, 2 * lref + 1.0) - lref);
        if (std::fabs(lgot - lref) > ulp) fail("rebuild loose", lref, lgot);
    }
    if (lgpu::df_to_double(DF{0.0f, 0.0f}) != 0.0) fail("rebuild zero", 0.0, 1.0);
    if (lgpu::df_to_double(DF{0.0f, 1.5f}) != 1.5) fail("rebuild lo only", 1.5, lgpu::df_to_double(DF{0.0f, 1.5f}));
    if (lgpu::df_to_double(DF{1.0f, -1.0f}) != 0.0) fail("rebuild cancel", 0.0, lgpu::df_to_double(DF{1.0f, -1.0f}));

    // bodies
    auto check_body = [&](int body, const double *m, double xr, double xi, double yr, double yi) {
        DF mdf[8];
        for (int k = 0; k < 8; k++) mdf[k] = lgpu::df_split_host(m[k]);
        double a = xr, b = xi, c = yr, d = yi;
        switch (body) {
        case 0: lgpu::body1_df<0>(mdf, a, b, c, d); break;
        case 1: lgpu::body1_df<1>(mdf, a, b, c, d); break;
        case 2: lgpu::body1_df<2>(mdf, a, b, c, d); break;
        case 3: lgpu::body1_df<3>(mdf, a, b, c, d); break;
        case 4: lgpu::body1_df<4>(mdf, a, b, c, d); break;
        default: lgpu::body1_df<5>(mdf, a, b, c, d); break;
        }
        // reference with the full matrix in long double (structured bodies
        // read only their own entries; the others are zero here)
        typedef long double L;
        const L m00r = m[0], m00i = m[1], m01r = m[2], m01i = m[3], m10r = m[4], m10i = m[5], m11r = m[6],
                m11i = m[7];
        L r0, i0, r1, i1;
        if (body == 5) {  // m00 = m11 = c, m01 = i u, m10 = i v
            r0 = m00r * xr - m01i * yi;
            i0 = m00r * xi + m01i * yr;
            r1 = m00r * yr - m10i * xi;
            i1 = m00r * yi + m10i * xr;
        } else if (body == 2) {
            r0 = yr;
            i0 = yi;
            r1 = xr;
            i1 = xi;
        } else {
            r0 = m00r * xr - m00i * xi + m01r * yr - m01i * yi;
            i0 = m00r * xi + m00i * xr + m01r * yi + m01i * yr;
            r1 = m10r * xr - m10i * xi + m11r * yr - m11i * yi;
            i1 = m10r * xi + m10i * xr + m11r * yi + m11i * yr;
        }
        const double scale = std::fmax(std::fmax(std::fabs(xr), std::fabs(xi)), std::fmax(std::fabs(yr), std::fabs(yi)));
        const double tol = 4e-14 * scale + 1e-300;
        n_body++;
        if (std::fabs(double(r0 - a)) > tol) fail("body re0", double(r0), a);
        if (std::fabs(double(i0 - b)) > tol) fail("body im0", double(i0), b);
        if (std::fabs(double(r1 - c)) > tol) fail("body re1", double(r1), c);
        if (std::fabs(double(i1 - d)) > tol) fail("body im1", double(i1), d);
    };
    std::uniform_int_distribution<int> amp_ex(-20, 0);
    for (int i = 0; i < 300000; i++) {
        const int body = i % 6;
        double m[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        // a random unitary-sized matrix with the body's structure
        const double th = 3.0 * u(gen), ph = 3.0 * u(gen), la = 3.0 * u(gen);
        const double c = std::cos(th), s = std::sin(th);
        if (body == 0) {
            m[0] = c; m[1] = 0; m[2] = -s * std::cos(la); m[3] = -s * std::sin(la);
            m[4] = s * std::cos(ph); m[5] = s * std::sin(ph); m[6] = c * std::cos(ph + la); m[7] = c * std::sin(ph + la);
        } else if (body == 1) {
            m[0] = std::cos(ph); m[1] = std::sin(ph); m[6] = std::cos(la); m[7] = std::sin(la);
        } else if (body == 3) {
            m[2] = std::cos(ph); m[3] = std::sin(ph); m[4] = std::cos(la); m[5] = std::sin(la);
        } else if (body == 4) {
            m[0] = c; m[2] = -s; m[4] = s; m[6] = c;
        } else if (body == 5) {
            m[0] = c; m[6] = c; m[3] = -s; m[5] = -s;
        }
        const double sc = std::ldexp(1.0, amp_ex(gen));
        check_body(body, m, sc * u(gen), sc * u(gen), sc * u(gen), sc * u(gen));
    }
    // NaN propagates
    {
        DF mdf[8];
        for (int k = 0; k < 8; k++) mdf[k] = lgpu::df_from_double(k == 0 ? std::nan("") : 0.5);
        double a = 0.3, b = 0.1, c = -0.2, d = 0.4;
        lgpu::body1_df<0>(mdf, a, b, c, d);
        if (!std::isnan(a)) fail("nan", a, a);
    }
    // conj(a) . (M a) over groups of 8 amplitudes (3-target expectations):
    // general complex M and amplitudes of mixed magnitudes, summed over 16
    // groups as the kernel does, against long double within 1e-13 of the
    // sum of |a|^2 |M|.
    long n_expval = 0;
    {
        std::uniform_int_distribution<int> aex(-14, 0);
        for (int trial = 0; trial < 2000; trial++) {
            double mm[128];
            DF mdf[128];
            double mscale = 0;
            for (int k = 0; k < 128; k++) {
                mm[k] = u(gen);
                mdf[k] = lgpu::df_from_double(mm[k]);
                mscale = std::max(mscale, std::fabs(mm[k]));
            }
            DF re{0.0f, 0.0f}, im{0.0f, 0.0f};
            long double rre = 0, rim = 0, norm = 0;
            for (int g = 0; g < 16; g++) {
                double a[16];
                DF ar[8], ai[8];
                for (int c = 0; c < 8; c++) {
                    const double sc = std::ldexp(1.0, aex(gen));
                    a[2 * c] = sc * u(gen);
                    a[2 * c + 1] = sc * u(gen);
                    ar[c] = lgpu::df_from_double(a[2 * c]);
                    ai[c] = lgpu::df_from_double(a[2 * c + 1]);
                    norm += (long double)a[2 * c] * a[2 * c] + (long double)a[2 * c + 1] * a[2 * c + 1];
                }
                lgpu::df_expval_group<8>(mdf, ar, ai, re, im);
                for (int r = 0; r < 8; r++) {
                    long double xr = 0, xi = 0;
                    for (int c = 0; c < 8; c++) {
                        const long double mr = mm[2 * (r * 8 + c)], mi = mm[2 * (r * 8 + c) + 1];
                        xr += mr * a[2 * c] - mi * a[2 * c + 1];
                        xi += mr * a[2 * c + 1] + mi * a[2 * c];
                    }
                    rre += a[2 * r] * xr + a[2 * r + 1] * xi;
                    rim += a[2 * r] * xi - a[2 * r + 1] * xr;
                }
            }
            const double bound = 1e-13 * double(norm) * mscale * 8;
            n_expval++;
            if (std::fabs(lgpu::df_to_double(re) - double(rre)) > bound) fail("expval re", lgpu::df_to_double(re), double(rre));
            if (std::fabs(lgpu::df_to_double(im) - double(rim)) > bound) fail("expval im", lgpu::df_to_double(im), double(rim));
        }
    }
    std::printf("split %ld rebuild %ld body %ld expval %ld bad %ld\n", n_split, n_rebuild, n_body, n_expval, bad);
    return bad == 0 ? 0 : 1;
}
