// host.cpp -- host-side inputs of the hot path, bit-exact with the reference:
// the seeded scatterer positions (Numerical Recipes "Ran" generator and the
// rejection sampler of the medium), the k-grids of the complex map and cut,
// and the Halton points that seed the resonance search.  Integer state and
// the same IEEE double operations in the same order give identical bits.
#include <cmath>
#include <cstdint>
#include "msgpu.h"
#include "error_text.h"

namespace {

// generator state (reference src/core/nru_random_type.h:349-354)
struct Ran {
    uint64_t u, v, w;

    // next_state (src/core/nru_random.c:24): LCG, xorshift, multiply-with-carry, combined
    uint64_t next() {
        u = u * 2862933555777941757ULL + 7046029254386353087ULL;
        v ^= v >> 17;
        v ^= v << 31;
        v ^= v >> 8;
        w = 4294957665ULL * (w & 0xffffffffULL) + (w >> 32);
        uint64_t x = u ^ (u << 21);
        x ^= x >> 35;
        x ^= x << 4;
        return (x + v) ^ w;
    }
    // random_double (nru_random.c:39): the 64-bit value times 2^-64
    double uniform() { return 5.42101086242752217E-20 * (double)next(); }
    // ratio-of-uniforms normal deviate (nru_random.c:48)
    double normal() {
        for (;;) {
            double a = uniform();
            double b = 1.7156 * (uniform() - 0.5);
            double x = a - 0.449871, y = std::fabs(b) + 0.386595;
            double q = x * x + y * (0.19600 * y - 0.25472 * x);
            if (q > 0.27597 && (q > 0.27846 || b * b > -4. * a * a * std::log(a))) continue;
            return b / a;
        }
    }
    // init_random (nru_random.c:63)
    explicit Ran(uint64_t seed) {
        v = 4101842887655102017ULL;
        w = 1;
        u = seed ^ v;
        next();
        v = u;
        next();
        w = v;
        next();
    }
};

double ball_volume(int d) {  // src/core/green_bessel.c:41
    if (d == 0) return 1.0;
    double vol = (d % 2 == 0) ? 3.1415926535897932385 : 2.0;
    for (int m = d; m > 2; m -= 2) vol *= 6.2831853071795864769 / m;
    return vol;
}

double halton(int i, int b) {  // src/core/domain_util.c:156
    double h = 0.0, f = 1.0;
    while (i > 0) {
        f /= b;
        h += f * (i % b);
        i /= b;
    }
    return h;
}

}  // namespace

extern "C" {

// fill_medium (src/core/medium_util.c:164-193) for the four shapes, then the
// volume-preserving stretch of the first coordinate when ratio != 1.
int msgpu_fill_medium(int d, int n, int shape, double ratio, uint64_t seed, double* pos) {
    if (d < 1 || d > 20 || n < 1 || !pos || ratio < 1.0)
        return msg::record_error(MSGPU_E_ARG, "fill_medium: bad argument (d in 1..20, n >= 1, ratio >= 1, pos)");
    Ran rng(seed);
    if (d == 1 && shape == MSGPU_BALL) shape = MSGPU_CUBE;
    const int ntot = n * d;
    switch (shape) {
    case MSGPU_CUBE: {
        double side = std::pow(n, 1.0 / d);
        for (int l = 0; l < ntot; l++) pos[l] = side * rng.uniform();
        break;
    }
    case MSGPU_BALL: {
        double rad = std::pow(n / ball_volume(d), 1.0 / d), r2 = rad * rad;
        for (int i = 0; i < n; i++) {
            double s2;
            do {
                s2 = 0.0;
                for (int c = 0; c < d; c++) {
                    double x = rad * (2 * rng.uniform() - 1);
                    pos[i * d + c] = x;
                    s2 += x * x;
                }
            } while (s2 > r2);
        }
        break;
    }
    case MSGPU_LATTICE: {
        int side = (int)std::ceil(std::pow(n, 1.0 / d));
        for (int i = 0; i < n; i++) {
            int v = i;
            for (int c = 0; c < d; c++) {
                pos[i * d + c] = v % side;
                v /= side;
            }
        }
        break;
    }
    case MSGPU_GAUSSIAN: {
        double sig = std::pow(n, 1.0 / d) / 2.506628274631000502;
        for (int l = 0; l < ntot; l++) pos[l] = sig * rng.normal();
        break;
    }
    default:
        return msg::record_error(MSGPU_E_ARG, "fill_medium: unknown shape");
    }
    if (ratio != 1.0 && d != 1) {
        double f2 = std::pow(ratio, -1.0 / d), f1 = ratio * f2;
        for (int l = 0; l < ntot; l++) pos[l] *= (l % d == 0) ? f1 : f2;
    }
    return 0;
}

// random_double (src/core/nru_random.c:39) n times from init_random(seed)
void msgpu_random_doubles(uint64_t seed, int n, double* out) {
    Ran rng(seed);
    for (int i = 0; i < n; i++) out[i] = rng.uniform();
}

// get_arg_cmap (src/core/complex_map_util.c:27-31): row-major from the top row
void msgpu_kplane_args(int nx, int ny, double xmin, double xmax, double ymin, double ymax, double* ks) {
    const double dx = (xmax - xmin) / (nx - 1), dy = (ymax - ymin) / (ny - 1);
    for (int l = 0; l < nx * ny; l++) {
        ks[2 * l] = xmin + (l % nx) * dx;
        ks[2 * l + 1] = ymax - (l / nx) * dy;
    }
}

// get_arg_ccut (src/core/complex_cut_util.c:32-36): triplets across the cut
// ((ns-il) zmin + (il-1) zmax)/(ns-1) + i dz (it-1), dz = (zmax-zmin)/(ns-1),
// in the reference's C99 complex arithmetic (real times complex is
// component-wise; i times dz swaps and negates).
void msgpu_kcut_args(int ns, const double* zmin, const double* zmax, double* ks) {
    const double dzr = (zmax[0] - zmin[0]) / (ns - 1), dzi = (zmax[1] - zmin[1]) / (ns - 1);
    for (int l = 0; l < 3 * (ns + 2); l++) {
        int il = l / 3, it = l % 3;
        double a = ns - il, b = il - 1;
        double re = (a * zmin[0] + b * zmax[0]) / (ns - 1);
        double im = (a * zmin[1] + b * zmax[1]) / (ns - 1);
        // I*dz*(it-1) = (-dzi, dzr) * (it-1)
        ks[2 * l] = re + (-dzi) * (it - 1);
        ks[2 * l + 1] = im + dzr * (it - 1);
    }
}

// the logarithmic mesh of init_logcut (src/core/log_cut_util.c:93-96):
// k_i = rek + i imkmin exp(ln(imkmax/imkmin) i / (ns-1)), the sample accumulating
// at rek as the mesh approaches the real axis
void msgpu_logcut_args(int ns, double rek, double imkmin, double imkmax, double* ks) {
    const double lfac = std::log(imkmax / imkmin);
    for (int i = 0; i < ns; i++) {
        ks[2 * i] = rek;
        ks[2 * i + 1] = imkmin * std::exp((lfac * i) / (ns - 1));
    }
}

// set_halton_points (src/core/domain_util.c:170-185), indices 1..n
void msgpu_halton_points(const double* dom, int n, double* z) {
    for (int i = 0; i < n; i++) {
        z[2 * i] = dom[0] + (dom[1] - dom[0]) * halton(i + 1, 2);
        z[2 * i + 1] = dom[2] + (dom[3] - dom[2]) * halton(i + 1, 3);
    }
}

}  // extern "C"
