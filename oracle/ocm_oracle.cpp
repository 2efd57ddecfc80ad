// ocm_oracle.cpp - TEST INFRASTRUCTURE, not part of the engine.
//
// FP64 CPU restatement of OpenCafeMol's hot-path force field, used only by
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
// checker.  It follows the reference's expression strings and parameter
// derivations and OpenMM 8.0.0's documented semantics:
//   harmonic bond          HarmonicBondForceFieldGenerator.cpp:3-14
//   Go 10-12 contact       GoContactForceFieldGenerator.cpp:3-20
//   flexible-local angle   FlexibleLocalAngleForceFieldGenerator.cpp:3-68,
//                          OpenMM Continuous1DFunction (natural cubic spline,
//                          zero outside [min, max])
//   flexible-local dihed.  FlexibleLocalDihedralForceFieldGenerator.cpp:5-62,
//                          reader selection ReadTOMLForceFieldGenerator.cpp:637-766
//                          (a GLY-PRO dihedral gets both the R2-PRO and the
//                          GLY-PRO series), IUPAC torsion sign
//   excluded volume        ExcludedVolumeForceFieldGenerator.cpp:23-92
//   Debye-Hueckel          DebyeHuckelForceFieldGenerator.hpp:36-41, .cpp:10-108
//   LJ repulsive/attract.  LennardJones{Repulsive,Attractive}ForceFieldGenerator.cpp,
//                          OpenMM switching 1 - 10x^3 + 15x^4 - 6x^5
//   exclusions             Topology.cpp:75-135 (ignore_list_within_edge)
//   participation          InteractionGroup.hpp:17-45 (value present)
//   Langevin               OpenMM LangevinIntegrator (leapfrog form)
//
// PARITY UNPINNED: the reference ships no golden vectors and its arithmetic
// lives in OpenMM, which is not available here; this restatement is pinned
// by analytic known-answer tests (tests/test_oracle.py) instead.
//
// Built with -ffp-contract=off: the FP32 cutoff emulation and the minimum
// scans must round exactly as written.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <functional>
#include <vector>

#include "oracle_system.h"
#include "oracle_tables.h"

namespace oracle {

constexpr double kPi = 3.1415926535897932385;
constexpr double kNa = 6.02214076e23;
constexpr double kKB = 1.380649e-23;
constexpr double kE = 1.6021766208e-19;
constexpr double kEps0 = 8.854187817e-12 * 1.0e3 * 1.0e-9 / kNa;
constexpr double kBoltz = 0.00831446261815324;  // kJ/mol/K
constexpr double kThetaMin = 1.30900, kThetaMax = 2.87979;

struct V3 {
    double x, y, z;
};
static inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 scale(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }

// ----------------------------------------------------------------------------
// Topology: exclusions within `dist` edges (depth-first walk that records a
// node before descending and never revisits a recorded node).
// ----------------------------------------------------------------------------
struct Graph {
    std::vector<std::vector<int64_t>> adj;
    explicit Graph(int64_t n) : adj(n) {}
    void add(int64_t a, int64_t b) {
        adj[a].push_back(b);
        adj[b].push_back(a);
    }
    void walk(int64_t node, int64_t dist, std::vector<int64_t>& out) const {
        out.push_back(node);
        if (dist == 0) return;
        for (int64_t m : adj[node])
            if (std::find(out.begin(), out.end(), m) == out.end()) walk(m, dist - 1, out);
    }
    std::vector<std::pair<int64_t, int64_t>> within(int64_t dist) const {
        std::vector<std::pair<int64_t, int64_t>> r;
        std::vector<int64_t> w;
        for (int64_t i = 0; i < (int64_t)adj.size(); ++i) {
            w.clear();
            walk(i, dist, w);
            for (int64_t j : w)
                if (j != i) r.emplace_back(std::min(i, j), std::max(i, j));
        }
        std::sort(r.begin(), r.end());
        r.erase(std::unique(r.begin(), r.end()), r.end());
        return r;
    }
};

// ----------------------------------------------------------------------------
// Flexible-local angle: OpenMM natural spline + the reference's minimum scan.
// ----------------------------------------------------------------------------
static void natural_spline(const double* y, double h, double* M) {
    // Solve M[k-1] + 4M[k] + M[k+1] = 6 (y[k+1] - 2y[k] + y[k-1]) / h^2,
    // M[0] = M[9] = 0, by Gaussian elimination of the tridiagonal system.
    double a[10] = {0}, rhs[10] = {0};
    for (int k = 1; k <= 8; ++k) rhs[k] = 6.0 * (y[k + 1] - 2.0 * y[k] + y[k - 1]) / (h * h);
    double diag[10];
    for (int k = 1; k <= 8; ++k) diag[k] = 4.0;
    for (int k = 2; k <= 8; ++k) {
        const double w = 1.0 / diag[k - 1];
        diag[k] -= w;
        rhs[k] -= w * rhs[k - 1];
    }
    M[0] = M[9] = 0.0;
    M[8] = rhs[8] / diag[8];
    for (int k = 7; k >= 1; --k) M[k] = (rhs[k] - M[k + 1]) / diag[k];
    (void)a;
}

static double fla_reference_interp(int aa, double th) {
    // The reference's own cubic with its rounded node list and its
    // second-derivative table (FlexibleLocalAngleForceFieldGenerator.cpp:47-68).
    static const double thetas[10] = {1.30900, 1.48353, 1.65806, 1.83260, 2.00713,
                                      2.18166, 2.35619, 2.53073, 2.70526, 2.87979};
    const double dtheta = (kThetaMax - kThetaMin) / 9.0;
    const double rdtheta = 1.0 / dtheta;
    constexpr double one_over_six = double(1.0) / double(6.0);
    std::size_t n = std::min<std::size_t>(8, (std::size_t)std::floor((th - kThetaMin) * rdtheta));
    if (thetas[n + 1] < th) n++;
    else if (th < thetas[n]) n--;
    const double a = (thetas[n + 1] - th) * rdtheta;
    const double b = (th - thetas[n]) * rdtheta;
    const double e1 = a * kFlaY[aa][n] + b * kFlaY[aa][n + 1];
    const double e2 = ((a * a * a - a) * kFlaD2[aa][n] + (b * b * b - b) * kFlaD2[aa][n + 1]) *
                      dtheta * dtheta * one_over_six;
    return e1 + e2;
}

static double fla_min_energy(int aa) {
    double m = kFlaY[aa][0];
    double th = kThetaMin;
    while (th < kThetaMax) {
        m = std::min(m, fla_reference_interp(aa, th));
        th += 1e-4;
    }
    return m;
}

static double fld_min_energy(const double* f) {
    double phi = -kPi, m = std::numeric_limits<double>::max();
    while (phi < kPi) {
        const double s1 = std::sin(phi), c1 = std::cos(phi);
        const double ss = s1 * s1, cc = c1 * c1;
        const double s2 = 2 * s1 * c1, c2 = cc - ss;
        const double s3 = s1 * (3 - 4 * ss), c3 = c1 * (4 * cc - 3);
        m = std::min(m, f[1] * c1 + f[2] * s1 + f[3] * c2 + f[4] * s2 + f[5] * c3 + f[6] * s3 + f[0]);
        phi += 1e-4;
    }
    return m;
}

// The scans above depend only on the table, so each runs once per process
// (thread-safe static initialisation).
static double fla_min_energy_cached(int aa) {
    static const std::vector<double> m = [] {
        std::vector<double> v(20);
        for (int a = 0; a < 20; ++a) v[a] = fla_min_energy(a);
        return v;
    }();
    return m[aa];
}

static double fld_min_energy_cached(int cls) {
    static const std::vector<double> m = [] {
        std::vector<double> v(23);
        for (int c = 0; c < 23; ++c) v[c] = fld_min_energy(kFld[c].c);
        return v;
    }();
    return m[cls];
}

// ----------------------------------------------------------------------------
// Debye-Hueckel parameters (DebyeHuckelForceFieldGenerator.cpp:22-46).
// ----------------------------------------------------------------------------
struct DHParams {
    double k_e, debye, cutoff, corr, eps_r;
};
static DHParams dh_params(double I, double T, double ratio) {
    DHParams p;
    p.eps_r = (249.4 - 0.788 * T + 7.2e-4 * T * T) *
              (1. - 2.551e-1 * I + 5.151e-2 * I * I - 6.889e-3 * I * I * I);
    const double eps0 = kEps0 / kE / kE;
    p.k_e = 1.0 / (4.0 * kPi * eps0 * p.eps_r);
    const double Ic = I * 1.0e-24;
    p.debye = std::sqrt((eps0 * p.eps_r * kKB * 1.0e-3 * T) / (2. * Ic));
    p.cutoff = p.debye * ratio;
    p.corr = std::exp(-ratio) / p.cutoff;
    return p;
}

// Largest and second largest present value, with the comparison the
// generator uses (strict for EXV, non-strict for LJ).
static std::pair<double, double> top_two(const double* v, int64_t n, bool strict) {
    double m1 = std::numeric_limits<double>::min(), m2 = std::numeric_limits<double>::min();
    for (int64_t i = 0; i < n; ++i) {
        if (std::isnan(v[i])) continue;
        const bool gt1 = strict ? (m1 < v[i]) : (m1 <= v[i]);
        const bool gt2 = strict ? (m2 < v[i]) : (m2 <= v[i]);
        if (gt1) {
            m2 = m1;
            m1 = v[i];
        } else if (gt2) {
            m2 = v[i];
        }
    }
    return {m1, m2};
}

// ----------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11) and Box-Muller normals: the same
// stream definition the engine uses.
// ----------------------------------------------------------------------------
static void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n1 = lo1, n2 = hi0 ^ c[3] ^ k1, n3 = lo0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}
static void gaussian3(uint32_t seed, uint32_t stream, uint32_t bead, uint64_t step, uint32_t purpose,
                      double g[3]) {
    uint32_t c[4] = {bead, (uint32_t)step, (uint32_t)(step >> 32), purpose};
    philox(c, seed, 0x6F636D31u ^ stream);
    double u[4];
    for (int k = 0; k < 4; ++k) u[k] = (double)((c[k] >> 8) + 1u) / 16777216.0;
    const double a = std::sqrt(-2.0 * std::log(u[0])), b = std::sqrt(-2.0 * std::log(u[2]));
    g[0] = a * std::cos(2.0 * kPi * u[1]);
    g[1] = a * std::sin(2.0 * kPi * u[1]);
    g[2] = b * std::cos(2.0 * kPi * u[3]);
}

}  // namespace oracle

using namespace oracle;

// Every unordered pair (i < j) closer than `cell` (minimum image when
// periodic) exactly once, found through a grid of cells at least `cell`
// wide.  Returns false (nothing visited) when a periodic box is narrower
// than three cells, where the all-pairs loop applies.
template <class Fn>
static bool cell_pairs(int64_t n, const V3* x, bool periodic, const double L[3], double cell, Fn&& fn) {
    double lo[3], ext[3];
    int nc[3];
    for (int c = 0; c < 3; ++c) {
        if (periodic) {
            lo[c] = 0;
            ext[c] = L[c];
        } else {
            double mn = 1e300, mx = -1e300;
            for (int64_t i = 0; i < n; ++i) {
                const double v = c == 0 ? x[i].x : (c == 1 ? x[i].y : x[i].z);
                mn = std::min(mn, v);
                mx = std::max(mx, v);
            }
            lo[c] = mn;
            ext[c] = mx - mn + 1e-9;
        }
        nc[c] = std::max(1, (int)std::floor(ext[c] / cell));
        if (periodic && nc[c] < 3) return false;
        nc[c] = std::min(nc[c], 1024);
    }
    const int64_t ncell = (int64_t)nc[0] * nc[1] * nc[2];
    std::vector<int64_t> head(ncell, -1), next(n, -1);
    std::vector<int> cidx(3 * n);
    for (int64_t i = 0; i < n; ++i) {
        const double v[3] = {x[i].x, x[i].y, x[i].z};
        int64_t lin = 0;
        for (int c = 0; c < 3; ++c) {
            double w = v[c] - lo[c];
            if (periodic) w -= L[c] * std::floor(w / L[c]);
            int k = (int)std::floor(w / ext[c] * nc[c]);
            k = std::min(nc[c] - 1, std::max(0, k));
            cidx[3 * i + c] = k;
            lin = lin * nc[c] + k;
        }
        next[i] = head[lin];
        head[lin] = i;
    }
    for (int64_t i = 0; i < n; ++i) {
        const int* ci = &cidx[3 * i];
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dz = -1; dz <= 1; ++dz) {
                    int k[3] = {ci[0] + dx, ci[1] + dy, ci[2] + dz};
                    bool ok = true;
                    int64_t lin = 0;
                    for (int c = 0; c < 3; ++c) {
                        if (periodic) k[c] = (k[c] + nc[c]) % nc[c];
                        else if (k[c] < 0 || k[c] >= nc[c]) ok = false;
                        lin = lin * nc[c] + k[c];
                    }
                    if (!ok) continue;
                    for (int64_t j = head[lin]; j >= 0; j = next[j])
                        if (j > i) fn(i, j);
                }
    }
    return true;
}

extern "C" {


// Energy slots: EXV, DH, LJR, LJA, HB, GO, FLA, FLD, GB, GD, capped Go.

int oracle_dh_params(double I, double T, double ratio, double* out5) {
    const DHParams p = dh_params(I, T, ratio);
    out5[0] = p.k_e;
    out5[1] = p.debye;
    out5[2] = p.cutoff;
    out5[3] = p.corr;
    out5[4] = p.eps_r;
    return 0;
}
double oracle_fla_min_energy(int aa) { return fla_min_energy_cached(aa); }
// Largest and second largest present value (strict comparison for EXV).
void oracle_top_two(const double* v, int64_t n, int strict, double* out2) {
    const auto t = top_two(v, n, strict != 0);
    out2[0] = t.first;
    out2[1] = t.second;
}
double oracle_fld_min_energy(int cls) { return fld_min_energy_cached(cls); }
int oracle_natural_spline(const double* y10, double h, double* M10) {
    natural_spline(y10, h, M10);
    return 0;
}
// Dihedral classes applied to a coef "A-B" (reference reader + map loop).
int oracle_fld_classes(int aa1, int aa2, int32_t* out, int cap) {
    int c = 0;
    const std::string a = kAA[aa1], b = kAA[aa2];
    for (int k = 0; k < 23; ++k) {
        const std::string f = kFld[k].first, s = kFld[k].second;
        bool take;
        if (s == "GLY") take = (b == "GLY");
        else if (s == "PRO") take = (f == "GLY") ? (a == "GLY" && b == "PRO") : (b == "PRO");
        else take = (b != "GLY" && b != "PRO" && a == f);
        if (take && c < cap) out[c++] = k;
    }
    return c;
}
int oracle_ignore_within(int64_t n, int64_t n_bond, const int64_t* bonds, int64_t n_contact,
                         const int64_t* contacts, int ign_bond, int ign_contact, int64_t* out,
                         int64_t cap, int64_t* n_out) {
    std::vector<std::pair<int64_t, int64_t>> r;
    if (ign_bond >= 0) {
        Graph g(n);
        for (int64_t k = 0; k < n_bond; ++k) g.add(bonds[2 * k], bonds[2 * k + 1]);
        auto v = g.within(ign_bond);
        r.insert(r.end(), v.begin(), v.end());
    }
    if (ign_contact >= 0) {
        Graph g(n);
        for (int64_t k = 0; k < n_contact; ++k) g.add(contacts[2 * k], contacts[2 * k + 1]);
        auto v = g.within(ign_contact);
        r.insert(r.end(), v.begin(), v.end());
    }
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
    *n_out = (int64_t)r.size();
    if ((int64_t)r.size() > cap) return 1;
    for (std::size_t k = 0; k < r.size(); ++k) {
        out[2 * k] = r[k].first;
        out[2 * k + 1] = r[k].second;
    }
    return 0;
}

int oracle_evaluate(const OracleSystem* s, double* forces, double* energies) {
    const int64_t n = s->n;
    std::vector<V3> x(n), f(n, V3{0, 0, 0});
    for (int64_t i = 0; i < n; ++i) x[i] = {s->pos[3 * i], s->pos[3 * i + 1], s->pos[3 * i + 2]};
    double E[11] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const double L[3] = {s->box[0], s->box[1], s->box[2]};
    auto min_image = [&](V3 d, bool per) {
        if (!per) return d;
        d.x -= L[0] * std::round(d.x / L[0]);
        d.y -= L[1] * std::round(d.y / L[1]);
        d.z -= L[2] * std::round(d.z / L[2]);
        return d;
    };
    auto add = [&](int64_t i, V3 v) {
        f[i].x += v.x;
        f[i].y += v.y;
        f[i].z += v.z;
    };

    // -------- bonds --------
    for (int64_t b = 0; b < s->n_bonds; ++b) {
        const int64_t i = s->bond_idx[2 * b], j = s->bond_idx[2 * b + 1];
        const V3 d = min_image(sub(x[j], x[i]), s->bond_periodic);
        const double r = std::sqrt(dot(d, d));
        const double dr = r - s->bond_v0[b];
        E[4] += 0.5 * s->bond_k[b] * dr * dr;
        const double sc = -s->bond_k[b] * dr / r;  // F_i = sc (x_i - x_j)
        add(i, scale(d, -sc));
        add(j, scale(d, sc));
    }
    // -------- Go contacts --------
    for (int64_t b = 0; b < s->n_go; ++b) {
        const int64_t i = s->go_idx[2 * b], j = s->go_idx[2 * b + 1];
        const V3 d = min_image(sub(x[j], x[i]), s->go_periodic);
        const double r = std::sqrt(dot(d, d));
        const double t = s->go_r0[b] / r;
        const double t10 = std::pow(t, 10), t12 = std::pow(t, 12);
        E[5] += s->go_k[b] * (5 * t12 - 6 * t10);
        const double dEdr = s->go_k[b] * (-60 * t12 + 60 * t10) / r;
        const double sc = -dEdr / r;
        add(i, scale(d, -sc));
        add(j, scale(d, sc));
    }
    // -------- capped Go contacts: linear below cap r0, Go 10-12 above --------
    if (s->n_cgo) {
        for (int64_t b = 0; b < s->n_cgo; ++b) {
            const double c = s->cgo_cap[b];
            const double slope = -60 * (std::pow(1 / c, 13.0) - std::pow(1 / c, 11.0));
            const double intercept = 65 * std::pow(1 / c, 12.0) - 66 * std::pow(1 / c, 10.0);
            const int64_t i = s->cgo_idx[2 * b], j = s->cgo_idx[2 * b + 1];
            const V3 d = min_image(sub(x[j], x[i]), s->cgo_periodic);
            const double r = std::sqrt(dot(d, d));
            const double r0 = s->cgo_r0[b], k = s->cgo_k[b];
            double dEdr;
            if (r / r0 <= c) {
                E[10] += k * (slope * r / r0 + intercept);
                dEdr = k * slope / r0;
            } else {
                const double t = r0 / r;
                const double t10 = std::pow(t, 10), t12 = std::pow(t, 12);
                E[10] += k * (5 * t12 - 6 * t10);
                dEdr = k * (-60 * t12 + 60 * t10) / r;
            }
            const double sc = -dEdr / r;
            add(i, scale(d, -sc));
            add(j, scale(d, sc));
        }
    }
    // -------- Gaussian bonds (GaussianBondForceFieldGenerator.cpp:5-7) --------
    for (int64_t b = 0; b < s->n_gb; ++b) {
        const int64_t i = s->gb_idx[2 * b], j = s->gb_idx[2 * b + 1];
        const V3 d = min_image(sub(x[j], x[i]), s->gb_periodic);
        const double r = std::sqrt(dot(d, d));
        const double dr = r - s->gb_v0[b];
        const double sg = s->gb_sigma[b];
        const double e = s->gb_k[b] * std::exp(-dr * dr / (2 * sg * sg));
        E[8] += e;
        const double dEdr = -e * dr / (sg * sg);
        const double sc = -dEdr / r;  // F_i = sc (x_i - x_j)
        add(i, scale(d, -sc));
        add(j, scale(d, sc));
    }
    // -------- flexible-local angles --------
    {
        double Mtab[20][10], emin[20];
        bool have[20] = {false};
        const double h = (kThetaMax - kThetaMin) / 9.0;
        for (int64_t a = 0; a < s->n_fla; ++a) {
            const int aa = s->fla_aa[a];
            if (!have[aa]) {
                natural_spline(kFlaY[aa], h, Mtab[aa]);
                emin[aa] = fla_min_energy_cached(aa);
                have[aa] = true;
            }
            const int64_t i1 = s->fla_idx[3 * a], i2 = s->fla_idx[3 * a + 1], i3 = s->fla_idx[3 * a + 2];
            const V3 u = sub(x[i1], x[i2]), v = sub(x[i3], x[i2]);
            const V3 nrm = cross(u, v);
            const double nl = std::sqrt(dot(nrm, nrm));
            const double th = std::atan2(nl, dot(u, v));
            double S, dS;
            if (th < kThetaMin) {
                S = 30.0 * (kThetaMin - th) + kFlaY[aa][0];
                dS = -30.0;
            } else if (th > kThetaMax) {
                S = 30.0 * (th - kThetaMax) + kFlaY[aa][9];
                dS = 30.0;
            } else {
                const double pos = (th - kThetaMin) / h;
                int k = std::min(8, std::max(0, (int)std::floor(pos)));
                const double B = pos - k, A = 1.0 - B;
                const double* y = kFlaY[aa];
                const double* M = Mtab[aa];
                S = A * y[k] + B * y[k + 1] + ((A * A * A - A) * M[k] + (B * B * B - B) * M[k + 1]) * h * h / 6.0;
                dS = (y[k + 1] - y[k]) / h + ((1 - 3 * A * A) * M[k] + (3 * B * B - 1) * M[k + 1]) * h / 6.0;
            }
            const double kk = s->fla_k[a];
            E[6] += kk * (S - emin[aa]);
            const double dE = kk * dS;
            const V3 un = cross(u, nrm), vn = cross(v, nrm);
            const V3 f1 = scale(un, -dE / (dot(u, u) * nl));
            const V3 f3 = scale(vn, dE / (dot(v, v) * nl));
            add(i1, f1);
            add(i3, f3);
            add(i2, V3{-f1.x - f3.x, -f1.y - f3.y, -f1.z - f3.z});
        }
    }
    // -------- flexible-local dihedrals --------
    {
        double emin[23];
        bool have[23] = {false};
        for (int64_t q = 0; q < s->n_fld; ++q) {
            int32_t cls[4];
            const int nc = oracle_fld_classes(s->fld_aa1[q], s->fld_aa2[q], cls, 4);
            const int64_t i1 = s->fld_idx[4 * q], i2 = s->fld_idx[4 * q + 1];
            const int64_t i3 = s->fld_idx[4 * q + 2], i4 = s->fld_idx[4 * q + 3];
            const V3 F = sub(x[i1], x[i2]), G = sub(x[i2], x[i3]), H = sub(x[i4], x[i3]);
            const V3 A = cross(F, G), B = cross(H, G);
            const double AA = dot(A, A), BB = dot(B, B), Gl = std::sqrt(dot(G, G));
            // IUPAC: phi = atan2(|b2| b1.(b2 x b3), (b1 x b2).(b2 x b3)),
            // b1 = x2 - x1 = -F, b2 = x3 - x2 = -G, b3 = x4 - x3 = H.
            const V3 b1 = scale(F, -1), b2 = scale(G, -1), b3 = H;
            const double phi = std::atan2(Gl * dot(b1, cross(b2, b3)), dot(cross(b1, b2), cross(b2, b3)));
            for (int c = 0; c < nc; ++c) {
                const double* t = kFld[cls[c]].c;
                if (!have[cls[c]]) {
                    emin[cls[c]] = fld_min_energy_cached(cls[c]);
                    have[cls[c]] = true;
                }
                const double kk = s->fld_k[q];
                E[7] += kk * (t[0] - emin[cls[c]] + t[1] * std::cos(phi) + t[2] * std::sin(phi) +
                              t[3] * std::cos(2 * phi) + t[4] * std::sin(2 * phi) +
                              t[5] * std::cos(3 * phi) + t[6] * std::sin(3 * phi));
                const double dE = kk * (-t[1] * std::sin(phi) + t[2] * std::cos(phi) -
                                        2 * t[3] * std::sin(2 * phi) + 2 * t[4] * std::cos(2 * phi) -
                                        3 * t[5] * std::sin(3 * phi) + 3 * t[6] * std::cos(3 * phi));
                const double ga = Gl / AA, gb = Gl / BB;
                const double fg = dot(F, G) / (AA * Gl), hg = dot(H, G) / (BB * Gl);
                const V3 d1 = scale(A, -ga), d4 = scale(B, gb);
                const V3 d2 = {(ga + fg) * A.x - hg * B.x, (ga + fg) * A.y - hg * B.y, (ga + fg) * A.z - hg * B.z};
                const V3 d3 = {-fg * A.x + (hg - gb) * B.x, -fg * A.y + (hg - gb) * B.y, -fg * A.z + (hg - gb) * B.z};
                add(i1, scale(d1, -dE));
                add(i2, scale(d2, -dE));
                add(i3, scale(d3, -dE));
                add(i4, scale(d4, -dE));
            }
        }
    }
    // -------- Gaussian dihedrals (GaussianDihedralForceFieldGenerator.cpp:5-12) --------
    for (int64_t q = 0; q < s->n_gd; ++q) {
        const int64_t i1 = s->gd_idx[4 * q], i2 = s->gd_idx[4 * q + 1];
        const int64_t i3 = s->gd_idx[4 * q + 2], i4 = s->gd_idx[4 * q + 3];
        const V3 F = min_image(sub(x[i1], x[i2]), s->gd_periodic);
        const V3 G = min_image(sub(x[i2], x[i3]), s->gd_periodic);
        const V3 H = min_image(sub(x[i4], x[i3]), s->gd_periodic);
        const V3 A = cross(F, G), B = cross(H, G);
        const double AA = dot(A, A), BB = dot(B, B), Gl = std::sqrt(dot(G, G));
        const V3 b1 = scale(F, -1), b2 = scale(G, -1), b3 = H;
        const double phi = std::atan2(Gl * dot(b1, cross(b2, b3)), dot(cross(b1, b2), cross(b2, b3)));
        const double pi = 3.1415926535897932385;
        double dt = phi - s->gd_theta0[q];
        dt -= std::floor((dt + pi) / (2 * pi)) * (2 * pi);
        const double sg = s->gd_sigma[q];
        const double e = s->gd_k[q] * std::exp(-dt * dt / (2 * sg * sg));
        E[9] += e;
        const double dE = -e * dt / (sg * sg);
        const double ga = Gl / AA, gb = Gl / BB;
        const double fg = dot(F, G) / (AA * Gl), hg = dot(H, G) / (BB * Gl);
        const V3 d1 = scale(A, -ga), d4 = scale(B, gb);
        const V3 d2 = {(ga + fg) * A.x - hg * B.x, (ga + fg) * A.y - hg * B.y, (ga + fg) * A.z - hg * B.z};
        const V3 d3 = {-fg * A.x + (hg - gb) * B.x, -fg * A.y + (hg - gb) * B.y, -fg * A.z + (hg - gb) * B.z};
        add(i1, scale(d1, -dE));
        add(i2, scale(d2, -dE));
        add(i3, scale(d3, -dE));
        add(i4, scale(d4, -dE));
    }
    // -------- pair terms --------
    std::vector<std::pair<int64_t, int64_t>> bond_edges, contact_edges;
    for (int64_t b = 0; b < s->n_bonds; ++b) bond_edges.emplace_back(s->bond_idx[2 * b], s->bond_idx[2 * b + 1]);
    for (int64_t b = 0; b < s->n_go; ++b) contact_edges.emplace_back(s->go_idx[2 * b], s->go_idx[2 * b + 1]);
    if (s->cgo_contact_edges)
        for (int64_t b = 0; b < s->n_cgo; ++b) contact_edges.emplace_back(s->cgo_idx[2 * b], s->cgo_idx[2 * b + 1]);
    struct Term {
        int on, kind;
        int ign_bond, ign_contact;
        double rc, rc2f_dummy;
        std::vector<std::pair<int64_t, int64_t>> excl;
    };
    Term T[4];
    T[0] = {s->exv_on, 0, s->exv_ign_bond, s->exv_ign_contact, 0, 0, {}};
    T[1] = {s->dh_on, 1, s->dh_ign_bond, s->dh_ign_contact, 0, 0, {}};
    T[2] = {s->ljr_on, 2, s->ljr_ign_bond, s->ljr_ign_contact, 0, 0, {}};
    T[3] = {s->lja_on, 3, s->lja_ign_bond, s->lja_ign_contact, 0, 0, {}};
    DHParams dh{};
    double exv_corr = 0, lja_rs = 0;
    if (s->exv_on) {
        auto t2 = top_two(s->exv_radius, n, true);
        T[0].rc = (t2.first + t2.second) * s->exv_ratio;
        exv_corr = std::pow(1.0 / T[0].rc, 12);
    }
    if (s->dh_on) {
        dh = dh_params(s->dh_I, s->dh_T, s->dh_ratio);
        T[1].rc = dh.cutoff;
    }
    if (s->ljr_on) {
        auto t2 = top_two(s->ljr_sigma, n, false);
        T[2].rc = (t2.first + t2.second) * 0.5 * s->ljr_ratio;
    }
    if (s->lja_on) {
        auto t2 = top_two(s->lja_sigma, n, false);
        T[3].rc = (t2.first + t2.second) * 0.5 * s->lja_ratio;
        lja_rs = 0.9 * T[3].rc;
    }
    std::vector<std::vector<uint8_t>> ex_bits_dummy;
    // exclusion bitmask per pair: map from (i, j) to term bits
    std::vector<std::vector<std::pair<int64_t, uint8_t>>> excl(n);
    for (int t = 0; t < 4; ++t) {
        if (!T[t].on) continue;
        std::vector<int64_t> eb, ec;
        for (auto& e : bond_edges) { eb.push_back(e.first); eb.push_back(e.second); }
        for (auto& e : contact_edges) { ec.push_back(e.first); ec.push_back(e.second); }
        std::vector<std::pair<int64_t, int64_t>> r;
        if (T[t].ign_bond >= 0) {
            Graph g(n);
            for (auto& e : bond_edges) g.add(e.first, e.second);
            auto v = g.within(T[t].ign_bond);
            r.insert(r.end(), v.begin(), v.end());
        }
        if (T[t].ign_contact >= 0) {
            Graph g(n);
            for (auto& e : contact_edges) g.add(e.first, e.second);
            auto v = g.within(T[t].ign_contact);
            r.insert(r.end(), v.begin(), v.end());
        }
        for (auto& p : r) {
            excl[p.first].emplace_back(p.second, (uint8_t)(1 << t));
        }
    }
    for (auto& v : excl) std::sort(v.begin(), v.end());
    auto excl_bits = [&](int64_t i, int64_t j) {
        uint8_t b = 0;
        auto& v = excl[i];
        auto it = std::lower_bound(v.begin(), v.end(), std::make_pair(j, (uint8_t)0));
        for (; it != v.end() && it->first == j; ++it) b |= it->second;
        return b;
    };
    // FP32 cutoff emulation (engine canonical form).
    std::vector<float> xf(3 * n);
    float Lf[3] = {(float)L[0], (float)L[1], (float)L[2]};
    float iLf[3] = {L[0] > 0 ? (float)(1.0 / L[0]) : 0.f, L[1] > 0 ? (float)(1.0 / L[1]) : 0.f,
                    L[2] > 0 ? (float)(1.0 / L[2]) : 0.f};
    for (int64_t i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c) {
            double w = s->pos[3 * i + c];
            if (s->periodic) {
                const double k = std::floor(w * (1.0 / L[c]));
                w = w - k * L[c];
            }
            xf[3 * i + c] = (float)w;
        }
    float rc2f[4];
    for (int t = 0; t < 4; ++t) rc2f[t] = (float)(T[t].rc * T[t].rc);
    const bool any_pair = s->exv_on || s->dh_on || s->ljr_on || s->lja_on;
    auto sides = [](const int8_t* side, int64_t i, int64_t j) {
        return !side || ((side[i] & 1) && (side[j] & 2)) || ((side[i] & 2) && (side[j] & 1));
    };
    // molecule of every bead (union-find over the bond edges), if any term asks
    std::vector<int64_t> mol;
    if (s->ign_molecule[0] || s->ign_molecule[1] || s->ign_molecule[2] || s->ign_molecule[3]) {
        mol.resize(n);
        for (int64_t i = 0; i < n; ++i) mol[i] = i;
        std::function<int64_t(int64_t)> root = [&](int64_t a) { return mol[a] == a ? a : (mol[a] = root(mol[a])); };
        for (auto& e : bond_edges) {
            const int64_t a = root(e.first), b = root(e.second);
            if (a != b) mol[std::max(a, b)] = std::min(a, b);
        }
        for (int64_t i = 0; i < n; ++i) mol[i] = root(i);
    }
    auto other_molecule = [&](int t, int64_t i, int64_t j) { return !s->ign_molecule[t] || mol[i] != mol[j]; };
    // true unless term t ignores the pair's (group, group) combination
    auto groups_ok = [&](int t, int64_t i, int64_t j) {
        if (!s->grp || s->n_igp[t] == 0) return true;
        const int32_t a = s->grp[i], b = s->grp[j];
        if (a < 0 || b < 0) return true;
        for (int64_t k = 0; k < s->n_igp[t]; ++k) {
            const int32_t p = s->igp[t][2 * k], q = s->igp[t][2 * k + 1];
            if ((p == a && q == b) || (p == b && q == a)) return false;
        }
        return true;
    };
    // One unordered pair (i < j): every pair term, exclusions and the
    // FP32 cutoff emulation; both enumerations below call it.
    auto pair = [&](int64_t i, int64_t j) {
                const V3 d = min_image(sub(x[j], x[i]), s->periodic);
                const double r2 = dot(d, d);
                const double r = std::sqrt(r2);
                float r2f = 0;
                if (s->fp32_cutoff) {
                    float dx = xf[3 * j] - xf[3 * i], dy = xf[3 * j + 1] - xf[3 * i + 1],
                          dz = xf[3 * j + 2] - xf[3 * i + 2];
                    if (s->periodic) {
                        dx = std::fmaf(-Lf[0], std::rint(dx * iLf[0]), dx);
                        dy = std::fmaf(-Lf[1], std::rint(dy * iLf[1]), dy);
                        dz = std::fmaf(-Lf[2], std::rint(dz * iLf[2]), dz);
                    }
                    r2f = std::fmaf(dz, dz, std::fmaf(dy, dy, dx * dx));
                }
                auto inside = [&](int t) {
                    return s->fp32_cutoff ? (r2f < rc2f[t]) : (r < T[t].rc);
                };
                const uint8_t eb = excl_bits(i, j);
                double sc = 0;  // F_i = sc (x_i - x_j)
                if (s->exv_on && !(eb & 1) && groups_ok(0, i, j) && other_molecule(0, i, j) && !std::isnan(s->exv_radius[i]) &&
                    !std::isnan(s->exv_radius[j]) && inside(0)) {
                    const double S = s->exv_radius[i] + s->exv_radius[j];
                    const double S12 = std::pow(S, 12);
                    E[0] += s->exv_eps * S12 * (std::pow(1.0 / r, 12) - exv_corr);
                    sc += 12.0 * s->exv_eps * S12 / std::pow(r, 14);
                }
                if (s->dh_on && !(eb & 2) && groups_ok(1, i, j) && other_molecule(1, i, j) && !std::isnan(s->dh_q[i]) && !std::isnan(s->dh_q[j]) &&
                    inside(1)) {
                    const double qq = s->dh_q[i] * s->dh_q[j] * dh.k_e;
                    const double ex = std::exp(-r / dh.debye);
                    E[1] += qq * (ex / r - dh.corr);
                    sc += qq * ex * (1.0 / dh.debye + 1.0 / r) / r2;
                }
                if (s->ljr_on && !(eb & 4) && groups_ok(2, i, j) && other_molecule(2, i, j) && !std::isnan(s->ljr_sigma[i]) &&
                    !std::isnan(s->ljr_sigma[j]) && sides(s->ljr_side, i, j) && inside(2)) {
                    const double sig = (s->ljr_sigma[i] + s->ljr_sigma[j]) * 0.5;
                    const double eps = s->ljr_geometric ? std::sqrt(s->ljr_eps[i] * s->ljr_eps[j])
                                                        : (s->ljr_eps[i] + s->ljr_eps[j]) * 0.5;
                    if (r <= sig * std::pow(2.0, 1.0 / 6.0)) {
                        const double s6 = std::pow(sig / r, 6), s12 = s6 * s6;
                        E[2] += eps * (4 * (s12 - s6) + 1);
                        sc += 24 * eps * (2 * s12 - s6) / r2;
                    }
                }
                if (s->lja_on && !(eb & 8) && groups_ok(3, i, j) && other_molecule(3, i, j) && !std::isnan(s->lja_sigma[i]) &&
                    !std::isnan(s->lja_sigma[j]) && sides(s->lja_side, i, j) && inside(3)) {
                    const double sig = (s->lja_sigma[i] + s->lja_sigma[j]) * 0.5;
                    const double eps = (s->lja_eps[i] + s->lja_eps[j]) * 0.5;
                    double e, dedr;
                    if (r < sig * std::pow(2.0, 1.0 / 6.0)) {
                        e = -eps;
                        dedr = 0;
                    } else {
                        const double s6 = std::pow(sig / r, 6), s12 = s6 * s6;
                        e = 4 * eps * (s12 - s6);
                        dedr = 4 * eps * (-12 * s12 + 6 * s6) / r;
                    }
                    if (r > lja_rs) {
                        const double w = T[3].rc - lja_rs;
                        const double xx = (r - lja_rs) / w;
                        const double sw = 1 - 10 * xx * xx * xx + 15 * xx * xx * xx * xx - 6 * std::pow(xx, 5);
                        const double dsw = (-30 * xx * xx + 60 * xx * xx * xx - 30 * xx * xx * xx * xx) / w;
                        dedr = dedr * sw + e * dsw;
                        e *= sw;
                    }
                    E[3] += e;
                    sc += -dedr / r;
                }
                if (sc != 0) {
                    add(i, scale(d, -sc));
                    add(j, scale(d, sc));
                }
    };
    if (any_pair) {
        double rcmax = 0;
        for (int t = 0; t < 4; ++t)
            if (T[t].on) rcmax = std::max(rcmax, T[t].rc);
        const bool want_cells = s->pair_cells > 0 || (s->pair_cells < 0 && n > 4096);
        if (!want_cells || !cell_pairs(n, x.data(), s->periodic, L, rcmax * 1.0001, pair)) {
            for (int64_t i = 0; i < n; ++i)
                for (int64_t j = i + 1; j < n; ++j) pair(i, j);
        }
    }
    if (forces)
        for (int64_t i = 0; i < n; ++i) {
            forces[3 * i] = f[i].x;
            forces[3 * i + 1] = f[i].y;
            forces[3 * i + 2] = f[i].z;
        }
    if (energies)
        for (int k = 0; k < 11; ++k) energies[k] = E[k];
    return 0;
}

// One OpenMM LangevinIntegrator step (leapfrog form) from the given forces:
//   v' = a v + (1-a)/gamma F/m + sqrt(kT (1 - a^2)/m) R,   x' = x + v' dt
int oracle_langevin_step(int64_t n, double* x, double* v, const double* f, const double* mass,
                         double T, double gamma, double dt, uint32_t seed, uint32_t stream,
                         uint64_t step) {
    const double a = std::exp(-gamma * dt);
    const double fs = gamma == 0 ? dt : (1 - a) / gamma;
    const double kT = kBoltz * T;
    for (int64_t i = 0; i < n; ++i) {
        if (!(mass[i] > 0)) continue;
        double g[3];
        gaussian3(seed, stream, (uint32_t)i, step, 0u, g);
        const double ns = std::sqrt(kT * (1 - a * a) / mass[i]);
        for (int c = 0; c < 3; ++c) {
            v[3 * i + c] = a * v[3 * i + c] + fs * f[3 * i + c] / mass[i] + ns * g[c];
            x[3 * i + c] += v[3 * i + c] * dt;
        }
    }
    return 0;
}

// CPU baseline: `steps` full steps (forces + Langevin) of one system.
int oracle_simulate(const OracleSystem* s0, double* x, double* v, const double* mass, double T,
                    double gamma, double dt, uint32_t seed, uint64_t step0, int64_t steps) {
    OracleSystem s = *s0;
    s.pos = x;
    std::vector<double> f(3 * s.n);
    for (int64_t k = 0; k < steps; ++k) {
        oracle_evaluate(&s, f.data(), nullptr);
        oracle_langevin_step(s.n, x, v, f.data(), mass, T, gamma, dt, seed, 0u, step0 + k);
    }
    return 0;
}

void oracle_gaussian3(uint32_t seed, uint32_t stream, uint32_t bead, uint64_t step,
                      uint32_t purpose, double* g3) {
    gaussian3(seed, stream, bead, step, purpose, g3);
}

}  // extern "C"
