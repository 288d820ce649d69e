// mpgen.cpp -- seeded synthetic Mille records for the benchmark workloads.
//
// Plays the role of pede's built-in test-data generators (pede -t,
// mptest1.f90 / mptest2.f90): tracks through a detector with known
// misalignments, written as Mille records (measured value, local and global
// derivatives, labels; layout of mille.f90:27-59, double precision).
//
// kind 1: planar telescope, 1D strips.  Layers at z = 10*l cm, `nmod`
//         modules of 2 cm along x per layer, one x shift per module
//         (label = l*nmod + m + 1), straight tracks x = a + b z with a
//         uniform over the module span (re-drawn until every layer is hit)
//         and b uniform in +-0.05.  Global derivative 1 for the hit module.
// kind 2: 12-layer barrel, `nmod` modules in total with 6 rigid-body
//         parameters each (labels 6*m+1 .. 6*m+6), linearised helices with
//         5 local parameters (curvature, phi0, d0, cot(theta), z0), 2D hits
//         measured in a stereo-rotated module frame so that every global
//         derivative is non-zero (one parameter group per module).
// kind 3: the kind-2 barrel with broken-line tracks: a random number of hits
//         (minHits..maxHits) and two kink angles per thin scatterer between
//         hits, local parameters 4 + 2*(nhit-2) (band structured).
//
// Random numbers: xoshiro256** seeded by splitmix64 (public-domain
// algorithms by Blackman & Vigna), Gaussian deviates by the Box-Muller
// transform.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/mpgpu.h"

namespace {

struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t z = seed;
        for (int i = 0; i < 4; ++i) {
            z += 0x9E3779B97F4A7C15ull;
            uint64_t x = z;
            x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
            x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
            s[i] = x ^ (x >> 31);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    }
    double uni() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double uni(double a, double b) { return a + (b - a) * uni(); }
    double gauss() {
        double u1 = uni(), u2 = uni();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

struct Writer {
    int64_t *recPtr; int32_t *inder; double *glder;
    int64_t nrec = 0, nw = 0;
    bool fill;
    void beginRecord() {   // (recPtr[nrec] was set by the previous record's end, or is 0)
        if (fill) { inder[nw] = 0; glder[nw] = 0.0; }
        nw++;
    }
    void endRecord() { nrec++; if (fill) recPtr[nrec] = nw; }
    void word(int32_t i, double d) {
        if (fill) { inder[nw] = i; glder[nw] = d; }
        nw++;
    }
    // one measurement: value, local derivatives (index 1..), sigma, globals
    void meas(double m, int nl, const int32_t *li, const double *ld, double sigma, int ng,
              const int32_t *gl, const double *gd) {
        word(0, m);
        for (int k = 0; k < nl; ++k) word(li[k], ld[k]);
        word(0, sigma);
        for (int k = 0; k < ng; ++k) word(gl[k], gd[k]);
    }
};

// ---------------------------------------------------------------- kind 1
// track t's own random stream when the tracks are generated in parallel
// (cfg.threads > 1): seeded from (seed, t), so that any range of tracks can
// be made on its own; otherwise every track continues the geometry's stream
Rng track_rng(uint64_t seed, int64_t t) { return Rng(seed * 0x9E3779B97F4A7C15ull + (uint64_t)t + 1ull); }

void gen_telescope(const mpgen_cfg &c, Writer &w, double *truth, int64_t t0, int64_t t1, bool perTrack) {
    Rng rngG(c.seed);
    const int nl = c.nlayers, nm = c.nmod;
    const double pitch = 2.0, span = pitch * nm;
    std::vector<double> shift((size_t)nl * nm);
    for (size_t i = 0; i < shift.size(); ++i) shift[i] = rngG.uni(-c.misal, c.misal);
    if (truth) for (size_t i = 0; i < shift.size(); ++i) truth[i] = shift[i];
    const double sig = c.sigma1;
    for (int64_t t = t0; t < t1; ++t) {
        Rng rngT = perTrack ? track_rng(c.seed, t) : Rng(0);
        Rng &rng = perTrack ? rngT : rngG;
        double a, b;
        for (;;) {
            a = rng.uni(0.0, span);
            b = rng.uni(-0.05, 0.05);
            double x0 = a, x1 = a + b * 10.0 * (nl - 1);
            if (x0 >= 0 && x0 < span && x1 >= 0 && x1 < span) break;
        }
        w.beginRecord();
        for (int l = 0; l < nl; ++l) {
            double z = 10.0 * l, x = a + b * z;
            int m = (int)(x / pitch);
            if (m >= nm) m = nm - 1;
            int32_t label = l * nm + m + 1;
            double noise = sig * rng.gauss();
            if (c.outlierFrac > 0 && rng.uni() < c.outlierFrac) noise += 20.0 * sig * rng.gauss();
            double meas = x + shift[(size_t)label - 1] + noise;
            int32_t li[2] = {1, 2};
            double ld[2] = {1.0, z};
            int32_t gl[1] = {label};
            double gd[1] = {1.0};
            w.meas(meas, 2, li, ld, sig, 1, gl, gd);
        }
        w.endRecord();
    }
}

// ---------------------------------------------------------------- barrel
struct Barrel {
    int nl = 12;
    std::vector<double> R, zmax;
    std::vector<int> nphi, nz, first;
    int nmod = 0;
    std::vector<double> mis;  // 6 per module
    void build(int total, Rng &rng, double misal) {
        static const double radii[12] = {5, 9, 14, 20, 27, 35, 44, 54, 65, 77, 90, 104};
        R.assign(radii, radii + 12);
        const int NZ = 8;
        int perZ = total / NZ;  // modules per z ring summed over layers
        double sumR = 0;
        for (double r : R) sumR += r;
        nphi.resize(nl); nz.assign(nl, NZ); zmax.resize(nl); first.resize(nl);
        int used = 0;
        for (int l = 0; l < nl; ++l) {
            nphi[l] = (int)std::floor(perZ * R[l] / sumR);
            if (nphi[l] < 3) nphi[l] = 3;
            used += nphi[l];
        }
        for (int l = nl - 1; used < perZ; l = (l == 0 ? nl - 1 : l - 1)) { nphi[l]++; used++; }
        nmod = 0;
        for (int l = 0; l < nl; ++l) {
            first[l] = nmod;
            nmod += nphi[l] * nz[l];
            zmax[l] = 2.2 * R[l] + 15.0;
        }
        mis.resize((size_t)nmod * 6);
        for (int m = 0; m < nmod; ++m) {
            for (int d = 0; d < 3; ++d) mis[(size_t)m * 6 + d] = rng.uni(-misal, misal);
            for (int d = 3; d < 6; ++d) mis[(size_t)m * 6 + d] = rng.uni(-misal, misal) * 1e-2;
        }
    }
};

const double kStereo = 0.1;  // rad, rotation of the measurement frame

// global derivatives of (u, v) for the 6 rigid-body parameters of a module
void rigid_derivs(double u, double v, double tu, double tv, double gu[6], double gv[6]) {
    gu[0] = -1.0; gu[1] = 0.0; gu[2] = tu; gu[3] = tu * v; gu[4] = -tu * u; gu[5] = -v;
    gv[0] = 0.0; gv[1] = -1.0; gv[2] = tv; gv[3] = tv * v; gv[4] = -tv * u; gv[5] = u;
}

void gen_barrel(const mpgen_cfg &c, Writer &w, double *truth, bool brokenLines, int64_t t0, int64_t t1,
                bool perTrack) {
    Rng rngG(c.seed);
    Barrel B;
    B.build(c.nmod, rngG, c.misal);
    if (truth) for (size_t i = 0; i < B.mis.size(); ++i) truth[i] = B.mis[i];
    const double cs = std::cos(kStereo), sn = std::sin(kStereo);
    const double bfield = 0.006;  // 0.3 * 2 T, in 1/(GeV cm) after / 100
    const double twopi = 6.283185307179586;
    std::vector<double> dp(2 + 4 + 2 * 64);
    for (int64_t t = t0; t < t1; ++t) {
        Rng rngT = perTrack ? track_rng(c.seed, t) : Rng(0);
        Rng &rng = perTrack ? rngT : rngG;
        // true track (for the hit positions)
        double pt = std::exp(rng.uni(std::log(1.0), std::log(100.0)));
        double q = rng.uni() < 0.5 ? -1.0 : 1.0;
        double kappa = q * bfield / pt;
        double phi0 = rng.uni(0.0, twopi);
        double lam = std::sinh(rng.uni(-1.5, 1.5));
        double d0 = 0.1 * rng.gauss(), z0 = 5.0 * rng.gauss();
        int nhit = B.nl;
        if (brokenLines) {
            nhit = c.minHits + (int)(rng.uni() * (c.maxHits - c.minHits + 1));
            if (nhit > c.maxHits) nhit = c.maxHits;
        }
        int nloc = brokenLines ? 4 + 2 * (nhit - 2) : 5;
        // corrections of the reference trajectory that the local fit determines
        if (!brokenLines) {
            dp[1] = 1e-5 * rng.gauss(); dp[2] = 1e-4 * rng.gauss(); dp[3] = 1e-2 * rng.gauss();
            dp[4] = 1e-4 * rng.gauss(); dp[5] = 1e-2 * rng.gauss();
        } else {
            dp[1] = 1e-2 * rng.gauss(); dp[2] = 1e-4 * rng.gauss();
            dp[3] = 1e-2 * rng.gauss(); dp[4] = 1e-4 * rng.gauss();
            for (int k = 5; k <= nloc; ++k) dp[k] = c.theta0 * rng.gauss();
        }
        w.beginRecord();
        double Rfirst = B.R[0];
        for (int h = 0; h < nhit; ++h) {
            int l = h % B.nl;
            double Rr = B.R[l] + (h / B.nl) * 1.0;
            double phi = phi0 + (d0 + kappa * Rr * Rr * 0.5) / Rr;
            double z = z0 + lam * Rr;
            double pw = twopi / B.nphi[l];
            double pn = std::fmod(phi, twopi);
            if (pn < 0) pn += twopi;
            int ip = (int)(pn / pw);
            if (ip >= B.nphi[l]) ip = B.nphi[l] - 1;
            double zl = B.zmax[l];
            int iz = (int)((z + zl) / (2.0 * zl / B.nz[l]));
            if (iz < 0) iz = 0;
            if (iz >= B.nz[l]) iz = B.nz[l] - 1;
            int mod = B.first[l] + iz * B.nphi[l] + ip;
            double phic = (ip + 0.5) * pw, zc = -zl + (iz + 0.5) * (2.0 * zl / B.nz[l]);
            double u = Rr * (pn - phic), v = z - zc;
            double tu = kappa * Rr - d0 / Rr, tv = lam;
            double gu[6], gv[6];
            rigid_derivs(u, v, tu, tv, gu, gv);
            const double *mis = &B.mis[(size_t)mod * 6];
            double lu[80], lv[80];
            int32_t li[80];
            int nl = 0;
            if (!brokenLines) {
                // (kappa, phi0, d0, cot theta, z0)
                double a[5] = {Rr * Rr * 0.5, Rr, 1.0, 0.0, 0.0};
                double b[5] = {0.0, 0.0, 0.0, Rr, 1.0};
                for (int k = 0; k < 5; ++k) { li[k] = k + 1; lu[k] = a[k]; lv[k] = b[k]; }
                nl = 5;
            } else {
                // offsets (u0, v0) and slopes at the first hit, kinks (ku_j,
                // kv_j) at the scatterers j = 1..nhit-2 between hits; a kink
                // reaches the hits that follow it up to two scatterers on
                double dR = Rr - Rfirst;
                li[nl] = 1; lu[nl] = 1.0; lv[nl] = 0.0; nl++;
                li[nl] = 2; lu[nl] = dR; lv[nl] = 0.0; nl++;
                li[nl] = 3; lu[nl] = 0.0; lv[nl] = 1.0; nl++;
                li[nl] = 4; lu[nl] = 0.0; lv[nl] = dR; nl++;
                int jlo = h - 2 >= 1 ? h - 2 : 1;
                for (int j = jlo; j <= h - 1 && j <= nhit - 2; ++j) {
                    int lj = j % B.nl;
                    double lever = Rr - (B.R[lj] + (j / B.nl) * 1.0);
                    li[nl] = 4 + 2 * j - 1; lu[nl] = lever; lv[nl] = 0.0; nl++;
                    li[nl] = 4 + 2 * j; lu[nl] = 0.0; lv[nl] = lever; nl++;
                }
            }
            double g1[6], g2[6];
            double r1 = 0.0, r2 = 0.0;
            for (int d = 0; d < 6; ++d) {
                g1[d] = cs * gu[d] + sn * gv[d];
                g2[d] = -sn * gu[d] + cs * gv[d];
                r1 += g1[d] * mis[d];
                r2 += g2[d] * mis[d];
            }
            int32_t i1[80], i2[80];
            double d1[80], d2[80];
            int n1l = 0, n2l = 0;
            for (int k = 0; k < nl; ++k) {
                double a1 = cs * lu[k] + sn * lv[k], a2 = -sn * lu[k] + cs * lv[k];
                if (a1 != 0.0) { i1[n1l] = li[k]; d1[n1l++] = a1; r1 += a1 * dp[li[k]]; }
                if (a2 != 0.0) { i2[n2l] = li[k]; d2[n2l++] = a2; r2 += a2 * dp[li[k]]; }
            }
            double e1 = c.sigma1 * rng.gauss(), e2 = c.sigma2 * rng.gauss();
            if (c.outlierFrac > 0 && rng.uni() < c.outlierFrac) e1 += 20.0 * c.sigma1 * rng.gauss();
            int32_t gl[6];
            for (int d = 0; d < 6; ++d) gl[d] = 6 * mod + d + 1;
            w.meas(r1 + e1, n1l, i1, d1, c.sigma1, 6, gl, g1);
            w.meas(r2 + e2, n2l, i2, d2, c.sigma2, 6, gl, g2);
        }
        if (brokenLines) {
            // kink pseudo-measurements: expectation 0, sigma theta0, local only
            for (int j = 1; j <= nhit - 2; ++j) {
                int32_t la[1] = {4 + 2 * j - 1}, lb[1] = {4 + 2 * j};
                double one[1] = {1.0};
                w.meas(0.0, 1, la, one, c.theta0, 0, nullptr, nullptr);
                w.meas(0.0, 1, lb, one, c.theta0, 0, nullptr, nullptr);
            }
        }
        w.endRecord();
    }
}

int run_range(const mpgen_cfg *c, Writer &w, double *truth, int64_t t0, int64_t t1, bool perTrack) {
    switch (c->kind) {
    case 1: gen_telescope(*c, w, truth, t0, t1, perTrack); return 0;
    case 2: gen_barrel(*c, w, truth, false, t0, t1, perTrack); return 0;
    case 3: gen_barrel(*c, w, truth, true, t0, t1, perTrack); return 0;
    default: return 24;
    }
}

// all tracks; with cfg.threads > 1 in ranges on that many threads (a
// counting pass per range gives each range its record and word offsets)
int run(const mpgen_cfg *c, Writer &w, double *truth) {
    if (!c) return 24;
    if (c->kind < 1 || c->kind > 3) return 24;
    const int nt = (int)std::min<int64_t>(std::max(c->threads, 1), std::max<int64_t>(c->ntracks / 1024, 1));
    if (nt <= 1) return run_range(c, w, truth, 0, c->ntracks, false);
    std::vector<int64_t> nr(nt + 1, 0), nwd(nt + 1, 0);
    auto range = [&](int i) { return std::make_pair(c->ntracks * i / nt, c->ntracks * (i + 1) / nt); };
    {
        std::vector<std::thread> th;
        for (int i = 0; i < nt; ++i)
            th.emplace_back([&, i] {
                Writer wc{nullptr, nullptr, nullptr};
                wc.fill = false;
                const auto r = range(i);
                run_range(c, wc, nullptr, r.first, r.second, true);
                nr[i + 1] = wc.nrec;
                nwd[i + 1] = wc.nw;
            });
        for (std::thread &t : th) t.join();
    }
    for (int i = 0; i < nt; ++i) { nr[i + 1] += nr[i]; nwd[i + 1] += nwd[i]; }
    if (!w.fill) {
        w.nrec = nr[nt];
        w.nw = nwd[nt];
        return 0;
    }
    std::vector<std::thread> th;
    for (int i = 0; i < nt; ++i)
        th.emplace_back([&, i] {
            Writer wf{w.recPtr, w.inder, w.glder};
            wf.fill = true;
            wf.nrec = nr[i];
            wf.nw = nwd[i];
            const auto r = range(i);
            run_range(c, wf, i == 0 ? truth : nullptr, r.first, r.second, true);
        });
    for (std::thread &t : th) t.join();
    w.nrec = nr[nt];
    w.nw = nwd[nt];
    return 0;
}

}  // namespace

extern "C" int mpgen_count(const mpgen_cfg *cfg, int64_t *nrec, int64_t *nwords,
                           int32_t *nlabels) {
    Writer w{nullptr, nullptr, nullptr};
    w.fill = false;
    int rc = run(cfg, w, nullptr);
    if (rc) return rc;
    *nrec = w.nrec;
    *nwords = w.nw;
    if (nlabels) {
        if (cfg->kind == 1) *nlabels = cfg->nlayers * cfg->nmod;
        else {
            Rng rng(cfg->seed);
            Barrel B;
            B.build(cfg->nmod, rng, cfg->misal);
            *nlabels = 6 * B.nmod;
        }
    }
    return 0;
}

extern "C" int mpgen_fill(const mpgen_cfg *cfg, int64_t *recPtr, int32_t *inder, double *glder,
                          double *truth) {
    Writer w{recPtr, inder, glder};
    w.fill = true;
    recPtr[0] = 0;
    return run(cfg, w, truth);
}

// Linear constraints removing the weak modes.
// kind 1: sum of shifts = 0 and sum of shift*z = 0 (z in units of 10 cm).
// kind 2/3: for each of the 6 rigid-body parameters: sum = 0, sum weighted
// by z/100, sum weighted by R/100 (18 constraints).
extern "C" int mpgen_constraints(const mpgen_cfg *cfg, int32_t *ncon, int32_t *conStart,
                                 int32_t *conLabel, double *conCoef) {
    if (cfg->kind == 1) {
        int n = cfg->nlayers * cfg->nmod, k = 0;
        *ncon = 2;
        if (!conStart) return 0;
        conStart[0] = 0;
        for (int i = 0; i < n; ++i) { conLabel[k] = i + 1; conCoef[k++] = 1.0; }
        conStart[1] = k;
        for (int i = 0; i < n; ++i) {
            int l = i / cfg->nmod;
            conLabel[k] = i + 1;
            conCoef[k++] = (double)l;
        }
        conStart[2] = k;
        return 0;
    }
    Rng rng(cfg->seed);
    Barrel B;
    B.build(cfg->nmod, rng, cfg->misal);
    *ncon = 18;
    if (!conStart) return 0;
    int k = 0, c = 0;
    conStart[0] = 0;
    for (int d = 0; d < 6; ++d) {
        for (int type = 0; type < 3; ++type) {
            for (int l = 0; l < B.nl; ++l) {
                double zl = B.zmax[l];
                for (int iz = 0; iz < B.nz[l]; ++iz) {
                    double zc = -zl + (iz + 0.5) * (2.0 * zl / B.nz[l]);
                    for (int ip = 0; ip < B.nphi[l]; ++ip) {
                        int mod = B.first[l] + iz * B.nphi[l] + ip;
                        double coef = type == 0 ? 1.0 : (type == 1 ? zc / 100.0 : B.R[l] / 100.0);
                        conLabel[k] = 6 * mod + d + 1;
                        conCoef[k++] = coef;
                    }
                }
            }
            conStart[++c] = k;
        }
    }
    return 0;
}

extern "C" int mpgen_constraint_words(const mpgen_cfg *cfg) {
    if (cfg->kind == 1) return 2 * cfg->nlayers * cfg->nmod;
    Rng rng(cfg->seed);
    Barrel B;
    B.build(cfg->nmod, rng, cfg->misal);
    return 18 * B.nmod;
}
