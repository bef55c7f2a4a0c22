// Seeded initial conditions (host side). Replaces the unseeded
// Renderer.makeSpheres (Astro/Renderer.swift:441-493) with reproducible sets:
// every random number comes from a counter-based Philox4x32-10 generator
// (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11) keyed by the seed, with the counter (particle, system, draw, 0), so
// any host produces the same particles in any order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/astro_cuda.h"

namespace {

struct Philox {
    uint32_t k0, k1;

    static void mulhilo(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
        const uint64_t p = (uint64_t)a * (uint64_t)b;
        *hi = (uint32_t)(p >> 32);
        *lo = (uint32_t)p;
    }

    // Ten rounds of the Philox-4x32 bijection (multipliers and Weyl key
    // increments as published).
    void block(const uint32_t in[4], uint32_t out[4]) const {
        uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
        uint32_t a = k0, b = k1;
        for (int r = 0; r < 10; ++r) {
            uint32_t hi0, lo0, hi1, lo1;
            mulhilo(0xD2511F53u, c0, &hi0, &lo0);
            mulhilo(0xCD9E8D57u, c2, &hi1, &lo1);
            const uint32_t n0 = hi1 ^ c1 ^ a, n1 = lo1, n2 = hi0 ^ c3 ^ b, n3 = lo0;
            c0 = n0;
            c1 = n1;
            c2 = n2;
            c3 = n3;
            a += 0x9E3779B9u;
            b += 0xBB67AE85u;
        }
        out[0] = c0;
        out[1] = c1;
        out[2] = c2;
        out[3] = c3;
    }
};

// A stream of uniforms in (0, 1) for one (seed, system, particle).
class Stream {
  public:
    Stream(uint64_t seed, uint32_t system, uint32_t particle)
        : ph_{(uint32_t)seed, (uint32_t)(seed >> 32)}, sys_(system), part_(particle) {}

    double uniform() {
        if (used_ >= 2) refill();
        const uint64_t hi = buf_[2 * used_], lo = buf_[2 * used_ + 1];
        ++used_;
        const uint64_t bits = ((hi << 32) | lo) >> 11;  // 53 bits
        return ((double)bits + 0.5) * (1.0 / 9007199254740992.0);
    }

    double normal() {
        const double u1 = uniform(), u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
    }

  private:
    void refill() {
        const uint32_t ctr[4] = {part_, sys_, draw_++, 0u};
        ph_.block(ctr, buf_);
        used_ = 0;
    }
    Philox ph_;
    uint32_t sys_, part_, draw_ = 0, used_ = 2;
    uint32_t buf_[4] = {0, 0, 0, 0};
};

void set_pm(PositionMass& p, double x, double y, double z, double m) {
    std::memset(&p, 0, sizeof(p));
    p.position[0] = (float)x;
    p.position[1] = (float)y;
    p.position[2] = (float)z;
    p.mass = (float)m;
}

void set_vr(VelocityRadius& v, double x, double y, double z, double r) {
    std::memset(&v, 0, sizeof(v));
    v.velocity[0] = (float)x;
    v.velocity[1] = (float)y;
    v.velocity[2] = (float)z;
    v.radius = (float)r;
}

void isotropic(Stream& s, double r, double* x, double* y, double* z) {
    const double cz = 2.0 * s.uniform() - 1.0, phi = 2.0 * M_PI * s.uniform();
    const double sz = std::sqrt(std::max(0.0, 1.0 - cz * cz));
    *x = r * sz * std::cos(phi);
    *y = r * sz * std::sin(phi);
    *z = r * cz;
}

// Plummer sphere by the Aarseth-Henon-Wielen (1974) recipe: radius from the
// inverted cumulative mass (cut at 99.9% of the mass), speed by von Neumann
// rejection from q^2 (1 - q^2)^(7/2) times the local escape speed. G = 1.
void plummer_particle(Stream& s, double a, double mass_total, double* p, double* v) {
    const double u = std::min(s.uniform(), 0.999);
    const double r = a / std::sqrt(std::pow(u, -2.0 / 3.0) - 1.0);
    isotropic(s, r, &p[0], &p[1], &p[2]);
    double q = 0.0;
    for (int it = 0; it < 1000; ++it) {
        q = s.uniform();
        const double y = 0.1 * s.uniform();
        if (y < q * q * std::pow(1.0 - q * q, 3.5)) break;
    }
    const double ve = std::sqrt(2.0 * mass_total / a) * std::pow(1.0 + r * r / (a * a), -0.25);
    isotropic(s, q * ve, &v[0], &v[1], &v[2]);
}

}  // namespace

extern "C" int astro_generate_ic(uint32_t kind, uint64_t seed, uint32_t system, uint32_t n,
                                 double p0, double p1, PositionMass* pm, VelocityRadius* vr,
                                 ColorType* ct) {
    if (!pm || !vr || n == 0) return ASTRO_ERR_INVALID_ARGUMENT;
    if (ct) std::memset(ct, 0, sizeof(ColorType) * n);
    switch (kind) {
        case ASTRO_IC_PLUMMER: {
            const double a = p0 > 0 ? p0 : 1.0, m = p1 > 0 ? p1 : 1.0;
            for (uint32_t i = 0; i < n; ++i) {
                Stream s(seed, system, i);
                double p[3], v[3];
                plummer_particle(s, a, m, p, v);
                set_pm(pm[i], p[0], p[1], p[2], m / n);
                set_vr(vr[i], v[0], v[1], v[2], 0.0);
            }
            break;
        }
        case ASTRO_IC_TWO_PLUMMER: {
            // Two spheres (a = 1, M = 0.5 each) at separation d = p0 (default
            // 10) on a parabolic relative orbit with pericentre 1: relative
            // speed sqrt(2 G M / d), angular momentum sqrt(2 G M q).
            const double d = p0 > 0 ? p0 : 10.0, mtot = 1.0, peri = 1.0;
            const double vrel = std::sqrt(2.0 * mtot / d), h = std::sqrt(2.0 * mtot * peri);
            const double vt = h / d, vr_ = -std::sqrt(std::max(0.0, vrel * vrel - vt * vt));
            const uint32_t n1 = n / 2;
            for (uint32_t i = 0; i < n; ++i) {
                Stream s(seed, system, i);
                double p[3], v[3];
                plummer_particle(s, 1.0, 0.5, p, v);
                const double sign = i < n1 ? -0.5 : 0.5;
                p[0] += sign * d;
                v[0] += sign * vr_;
                v[1] += sign * vt;
                set_pm(pm[i], p[0], p[1], p[2], 1.0 / n);
                set_vr(vr[i], v[0], v[1], v[2], 0.0);
            }
            break;
        }
        case ASTRO_IC_DISK_BULGE: {
            // Exponential disk (R_d = 1, sech^2 height z_d = 0.1, 80% of the
            // mass) plus a Hernquist bulge (a_b = 0.2, 20%, cut at 99% of its
            // mass). Disk particles orbit at the circular speed of the
            // enclosed mass (spherical estimate); bulge particles get an
            // isotropic Gaussian speed with sigma^2 = G M(<r) / (3 r).
            const uint32_t nd = (uint32_t)std::llround(0.8 * n);
            const double m = 1.0 / n, rd = 1.0, zd = 0.1, ab = 0.2;
            std::vector<double> r(n);
            for (uint32_t i = 0; i < n; ++i) {
                Stream s(seed, system, i);
                double x, y, z;
                if (i < nd) {
                    const double R = -rd * std::log(s.uniform() * s.uniform());
                    const double phi = 2.0 * M_PI * s.uniform();
                    z = zd * std::atanh(std::min(0.999999, std::max(-0.999999, 2.0 * s.uniform() - 1.0)));
                    x = R * std::cos(phi);
                    y = R * std::sin(phi);
                } else {
                    const double su = std::sqrt(std::min(s.uniform(), 0.99));
                    isotropic(s, ab * su / (1.0 - su), &x, &y, &z);
                }
                set_pm(pm[i], x, y, z, m);
                r[i] = std::sqrt(x * x + y * y + z * z);
            }
            std::vector<uint32_t> order(n);
            for (uint32_t i = 0; i < n; ++i) order[i] = i;
            std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return r[a] < r[b]; });
            std::vector<double> menc(n);
            for (uint32_t k = 0; k < n; ++k) menc[order[k]] = (k + 1) * m;
            for (uint32_t i = 0; i < n; ++i) {
                Stream s(seed, system ^ 0x80000000u, i);
                const double x = pm[i].position[0], y = pm[i].position[1];
                const double rr = std::max(r[i], 1e-6);
                if (i < nd) {
                    const double R = std::max(std::sqrt(x * x + y * y), 1e-6);
                    const double vc = std::sqrt(menc[i] / rr) * std::sqrt(R / rr);
                    const double disp = 0.05 * vc;
                    set_vr(vr[i], -vc * y / R + disp * s.normal(), vc * x / R + disp * s.normal(),
                           disp * s.normal(), 0.0);
                } else {
                    const double sig = std::sqrt(menc[i] / (3.0 * rr));
                    set_vr(vr[i], sig * s.normal(), sig * s.normal(), sig * s.normal(), 0.0);
                }
            }
            break;
        }
        case ASTRO_IC_UNIFORM_CUBE: {
            // Unit cube, Gaussian velocities (sigma = p0, default 0.1),
            // log-normal masses (sigma = p1, default 0.5) normalised to 1.
            const double sv = p0 > 0 ? p0 : 0.1, sm = p1 > 0 ? p1 : 0.5;
            std::vector<double> mass(n);
            double total = 0.0;
            for (uint32_t i = 0; i < n; ++i) {
                Stream s(seed, system, i);
                const double x = s.uniform(), y = s.uniform(), z = s.uniform();
                mass[i] = std::exp(sm * s.normal());
                total += mass[i];
                set_pm(pm[i], x, y, z, 0.0);
                set_vr(vr[i], sv * s.normal(), sv * s.normal(), sv * s.normal(), 0.0);
            }
            for (uint32_t i = 0; i < n; ++i) pm[i].mass = (float)(mass[i] / total);
            break;
        }
        case ASTRO_IC_REFERENCE_SCENE: {
            // Renderer.swift:25-46,441-493: stars (type 0, mass 1e4, radius
            // 5e4, box +-1.3e6), planets (type 1, 1e3, 1e4, +-2e6), dust
            // (type 2, 1, 2, +-2e6); velocities uniform in +-2e4.
            const uint32_t nstars = (uint32_t)p0, nplanets = (uint32_t)p1;
            for (uint32_t i = 0; i < n; ++i) {
                Stream s(seed, system, i);
                uint32_t type;
                double mass, radius, factor;
                if (i < nstars) {
                    type = 0;
                    mass = 1e4;
                    radius = 5e4;
                    factor = 1.3;
                } else if (i < nstars + nplanets) {
                    type = 1;
                    mass = 1e3;
                    radius = 1e4;
                    factor = 2.0;
                } else {
                    type = 2;
                    mass = 1.0;
                    radius = 2.0;
                    factor = 2.0;
                }
                const double b = 1e6 * factor;
                const double x = (2 * s.uniform() - 1) * b, y = (2 * s.uniform() - 1) * b,
                             z = (2 * s.uniform() - 1) * b;
                set_pm(pm[i], x, y, z, mass);
                set_vr(vr[i], (2 * s.uniform() - 1) * 2e4, (2 * s.uniform() - 1) * 2e4,
                       (2 * s.uniform() - 1) * 2e4, radius);
                if (ct) {
                    ct[i].type = type;
                    ct[i].color[3] = type == 2 ? 0.0f : 1.0f;
                    if (type == 0) ct[i].color[0] = ct[i].color[1] = ct[i].color[2] = 1.0f;
                }
            }
            break;
        }
        default:
            return ASTRO_ERR_INVALID_ARGUMENT;
    }
    return ASTRO_OK;
}

extern "C" int astro_generate_system_sizes(uint64_t seed, uint32_t nsys, uint32_t n_min,
                                           uint32_t n_max, double a_min, double a_max,
                                           uint32_t* sizes, double* scales) {
    if (!sizes || nsys == 0 || n_min == 0 || n_max < n_min) return ASTRO_ERR_INVALID_ARGUMENT;
    const double lo = std::log((double)n_min), hi = std::log((double)n_max + 1.0);
    for (uint32_t s = 0; s < nsys; ++s) {
        Stream st(seed, 0xFFFFFFFFu, s);
        const double v = std::exp(lo + (hi - lo) * st.uniform());
        sizes[s] = std::min<uint32_t>(n_max, std::max<uint32_t>(n_min, (uint32_t)v));
        const double u = st.uniform();
        if (scales) scales[s] = a_min + (a_max - a_min) * u;
    }
    return ASTRO_OK;
}
