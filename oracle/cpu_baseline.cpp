// cpu_baseline.cpp - TEST INFRASTRUCTURE, not part of the engine.
//
// The timed CPU baseline: an FP32 restatement of the same force field and
// Langevin integrator as the FP64 oracle (ocm_oracle.cpp), written the way
// a CPU MD code runs it, so that the GPU numbers are compared with a fair
// CPU implementation and not with the all-pairs checker:
//   * FP32 pair and bonded arithmetic, FP32 positions and velocities;
//   * a Verlet half list (each pair once, Newton's third law) with a 0.3 nm
//     skin, built through a cell grid and rebuilt when a bead has moved more
//     than half the skin since the last build;
//   * OpenMP over independent systems (an ensemble), largest first, one
//     system per thread at a time.
// Terms: harmonic bonds, Go 10-12 contacts, flexible-local angles and
// dihedrals (with the GLY-PRO double count), excluded volume, Debye-Hueckel
// and the HPS Lennard-Jones pair with its switch - the expressions the
// oracle restates (reference files cited there).  Interaction groups,
// side lists, molecule and group ignores are refused (not needed by the
// timed workloads).  It is a reported baseline, not the reference: OpenMM,
// which holds the reference's arithmetic, is not installed.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <omp.h>

#include "oracle_system.h"
#include "oracle_tables.h"

namespace {

using oracle::kFlaY;
using oracle::kFld;

constexpr double kBoltz = 0.00831446261815324;  // kJ/mol/K
constexpr float kSkin = 0.3f;                    // nm
constexpr double kThetaMin = 1.30900, kThetaMax = 2.87979;

struct Fla {
    int32_t i, j, k;
    float kk;
    int32_t table;
};
struct Fld {
    int32_t i, j, k, l;
    float kk;
    int32_t table;  // one entry per applied Fourier class
};
struct Pair2 {
    int32_t i, j;
    float a, b;  // bond: r0, k ; Go: k, r0
};
struct Table {
    float y[10], m[10], emin;  // m = M h^2 / 6
};
struct Fourier {
    float c[7], emin;
};

struct CpuSystem {
    int64_t n = 0;
    bool periodic = false, bond_pbc = false, go_pbc = false;  // minimum image for pairs, bonds, contacts
    float box[3] = {0, 0, 0};
    std::vector<float> x, y, z, vx, vy, vz, fx, fy, fz, im;
    std::vector<float> rx, ry, rz;  // positions at the last list build
    std::vector<Pair2> bonds, go;
    std::vector<Fla> fla;
    std::vector<Fld> fld;
    std::vector<Table> fla_tab;
    std::vector<Fourier> fld_tab;
    // pair terms
    bool exv = false, dh = false, ljr = false, lja = false;
    float exv_eps = 0, exv_rc2 = 0, exv_corr = 0;
    float dh_k = 0, dh_il = 0, dh_rc2 = 0, dh_corr = 0;
    float ljr_rc2 = 0, lja_rc2 = 0, lja_rs = 0, lja_iw = 0;
    std::vector<float> rad, q, ljr_eps, ljr_sig, lja_eps, lja_sig;
    float list_rc2 = 0, list_rc = 0, pair_rc2 = 0;  // pair_rc2: the largest cutoff^2
    // exclusions: per bead i, sorted (j > i, term bits)
    std::vector<int32_t> ex_start, ex_j;
    std::vector<uint8_t> ex_bits;
    // Verlet half list
    std::vector<int32_t> nb_start, nb_j;
    std::vector<uint8_t> nb_bits;
    // Langevin
    float vscale = 0, fscale = 0, noise = 0, dt = 0;
    uint32_t seed = 0;
    uint64_t step = 0;
    int64_t builds = 0;
    double energy[4 + 4] = {0};
};

inline float min_image(float d, float L, float iL) { return L > 0 ? d - L * std::rint(d * iL) : d; }

// Philox4x32-10 (Salmon et al., SC'11): the same counter layout as the
// engine and the oracle, with FP32 Box-Muller normals.
inline void gaussian3f(uint32_t seed, uint32_t bead, uint64_t step, float g[3]) {
    uint32_t c[4] = {bead, (uint32_t)step, (uint32_t)(step >> 32), 0u};
    uint32_t k0 = seed, k1 = 0x6F636D31u;
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        c[1] = (uint32_t)p1;
        c[3] = (uint32_t)p0;
        c[0] = n0;
        c[2] = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    float u[4];
    for (int k = 0; k < 4; ++k) u[k] = (float)((c[k] >> 8) + 1u) * (1.0f / 16777216.0f);
    const float a = std::sqrt(-2.f * std::log(u[0])), b = std::sqrt(-2.f * std::log(u[2]));
    const float tp = 6.2831853f;
    g[0] = a * std::cos(tp * u[1]);
    g[1] = a * std::sin(tp * u[1]);
    g[2] = b * std::cos(tp * u[3]);
}

void build_list(CpuSystem& s) {
    const int64_t n = s.n;
    const float rc = s.list_rc;
    float lo[3], ext[3];
    int nc[3];
    const float* P[3] = {s.x.data(), s.y.data(), s.z.data()};
    bool cells = true;
    for (int c = 0; c < 3; ++c) {
        if (s.periodic) {
            lo[c] = 0.f;
            ext[c] = s.box[c];
        } else {
            float mn = 1e30f, mx = -1e30f;
            for (int64_t i = 0; i < n; ++i) {
                mn = std::min(mn, P[c][i]);
                mx = std::max(mx, P[c][i]);
            }
            lo[c] = mn;
            ext[c] = mx - mn + 1e-6f;
        }
        nc[c] = std::max(1, std::min(512, (int)std::floor(ext[c] / rc)));
        if (s.periodic && nc[c] < 3) cells = false;
    }
    s.nb_start.assign(n + 1, 0);
    s.nb_j.clear();
    s.nb_bits.clear();
    const float bx = s.box[0], by = s.box[1], bz = s.box[2];
    const float ibx = bx > 0 ? 1.f / bx : 0.f, iby = by > 0 ? 1.f / by : 0.f, ibz = bz > 0 ? 1.f / bz : 0.f;
    auto consider = [&](int64_t i, int64_t j) {
        float dx = s.x[j] - s.x[i], dy = s.y[j] - s.y[i], dz = s.z[j] - s.z[i];
        if (s.periodic) {
            dx = min_image(dx, bx, ibx);
            dy = min_image(dy, by, iby);
            dz = min_image(dz, bz, ibz);
        }
        if (dx * dx + dy * dy + dz * dz >= s.list_rc2) return;
        uint8_t bits = 0;
        const int32_t* b = s.ex_j.data() + s.ex_start[i];
        const int32_t* e = s.ex_j.data() + s.ex_start[i + 1];
        const int32_t* it = std::lower_bound(b, e, (int32_t)j);
        if (it != e && *it == j) bits = s.ex_bits[it - s.ex_j.data()];
        s.nb_j.push_back((int32_t)j);
        s.nb_bits.push_back(bits);
    };
    if (!cells) {
        for (int64_t i = 0; i < n; ++i) {
            for (int64_t j = i + 1; j < n; ++j) consider(i, j);
            s.nb_start[i + 1] = (int32_t)s.nb_j.size();
        }
    } else {
        const int64_t ncell = (int64_t)nc[0] * nc[1] * nc[2];
        std::vector<int32_t> cell(n), cstart(ncell + 1, 0), order(n);
        std::vector<int32_t> ci(3 * n);
        for (int64_t i = 0; i < n; ++i) {
            int64_t lin = 0;
            for (int c = 0; c < 3; ++c) {
                float w = P[c][i] - lo[c];
                if (s.periodic) w -= s.box[c] * std::floor(w / s.box[c]);
                int k = (int)std::floor(w / ext[c] * nc[c]);
                k = std::min(nc[c] - 1, std::max(0, k));
                ci[3 * i + c] = k;
                lin = lin * nc[c] + k;
            }
            cell[i] = (int32_t)lin;
            ++cstart[lin + 1];
        }
        for (int64_t c = 0; c < ncell; ++c) cstart[c + 1] += cstart[c];
        {
            std::vector<int32_t> fill(cstart.begin(), cstart.end() - 1);
            for (int64_t i = 0; i < n; ++i) order[fill[cell[i]]++] = (int32_t)i;  // increasing i per cell
        }
        std::vector<int32_t> cand;
        for (int64_t i = 0; i < n; ++i) {
            cand.clear();
            for (int dx = -1; dx <= 1; ++dx)
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dz = -1; dz <= 1; ++dz) {
                        int k[3] = {ci[3 * i] + dx, ci[3 * i + 1] + dy, ci[3 * i + 2] + dz};
                        bool ok = true;
                        int64_t lin = 0;
                        for (int c = 0; c < 3; ++c) {
                            if (s.periodic) k[c] = (k[c] + nc[c]) % nc[c];
                            else if (k[c] < 0 || k[c] >= nc[c]) ok = false;
                            lin = lin * nc[c] + k[c];
                        }
                        if (!ok) continue;
                        for (int32_t p = cstart[lin]; p < cstart[lin + 1]; ++p)
                            if (order[p] > i) cand.push_back(order[p]);
                    }
            std::sort(cand.begin(), cand.end());
            cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
            for (int32_t j : cand) consider(i, j);
            s.nb_start[i + 1] = (int32_t)s.nb_j.size();
        }
    }
    s.rx = s.x;
    s.ry = s.y;
    s.rz = s.z;
    ++s.builds;
}

// Forces (and energies when asked) of the current positions.
void forces(CpuSystem& s, bool energy) {
    const int64_t n = s.n;
    std::fill(s.fx.begin(), s.fx.end(), 0.f);
    std::fill(s.fy.begin(), s.fy.end(), 0.f);
    std::fill(s.fz.begin(), s.fz.end(), 0.f);
    double E[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    float* fx = s.fx.data();
    float* fy = s.fy.data();
    float* fz = s.fz.data();
    const float* X = s.x.data();
    const float* Y = s.y.data();
    const float* Z = s.z.data();
    const float bx = s.box[0], by = s.box[1], bz = s.box[2];
    const float ibx = bx > 0 ? 1.f / bx : 0.f, iby = by > 0 ? 1.f / by : 0.f, ibz = bz > 0 ? 1.f / bz : 0.f;
    // harmonic bonds and Go contacts
    for (const Pair2& b : s.bonds) {
        float dx = X[b.j] - X[b.i], dy = Y[b.j] - Y[b.i], dz = Z[b.j] - Z[b.i];
        if (s.bond_pbc) {
            dx = min_image(dx, bx, ibx);
            dy = min_image(dy, by, iby);
            dz = min_image(dz, bz, ibz);
        }
        const float r = std::sqrt(dx * dx + dy * dy + dz * dz);
        const float dr = r - b.a;
        const float sc = b.b * dr / r;  // F_i = sc d
        fx[b.i] += sc * dx; fy[b.i] += sc * dy; fz[b.i] += sc * dz;
        fx[b.j] -= sc * dx; fy[b.j] -= sc * dy; fz[b.j] -= sc * dz;
        if (energy) E[4] += 0.5f * b.b * dr * dr;
    }
    for (const Pair2& b : s.go) {
        float dx = X[b.j] - X[b.i], dy = Y[b.j] - Y[b.i], dz = Z[b.j] - Z[b.i];
        if (s.go_pbc) {
            dx = min_image(dx, bx, ibx);
            dy = min_image(dy, by, iby);
            dz = min_image(dz, bz, ibz);
        }
        const float r2 = dx * dx + dy * dy + dz * dz;
        const float t2 = b.b * b.b / r2;
        const float t10 = t2 * t2 * t2 * t2 * t2;
        const float sc = -60.f * b.a * t10 * (t2 - 1.f) / r2;  // F_i = sc d
        fx[b.i] += sc * dx; fy[b.i] += sc * dy; fz[b.i] += sc * dz;
        fx[b.j] -= sc * dx; fy[b.j] -= sc * dy; fz[b.j] -= sc * dz;
        if (energy) E[5] += b.a * t10 * (5.f * t2 - 6.f);
    }
    // flexible-local angles (natural spline, linear walls)
    const float h = (float)((kThetaMax - kThetaMin) / 9.0), ih = 1.f / h;
    for (const Fla& a : s.fla) {
        const Table& t = s.fla_tab[a.table];
        const float ux = X[a.i] - X[a.j], uy = Y[a.i] - Y[a.j], uz = Z[a.i] - Z[a.j];
        const float vx = X[a.k] - X[a.j], vy = Y[a.k] - Y[a.j], vz = Z[a.k] - Z[a.j];
        const float nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
        const float nl = std::sqrt(std::max(nx * nx + ny * ny + nz * nz, 1e-30f));
        const float th = std::atan2(nl, ux * vx + uy * vy + uz * vz);
        float S, dS;
        if (th < (float)kThetaMin) {
            S = 30.f * ((float)kThetaMin - th) + t.y[0];
            dS = -30.f;
        } else if (th > (float)kThetaMax) {
            S = 30.f * (th - (float)kThetaMax) + t.y[9];
            dS = 30.f;
        } else {
            const float pos = (th - (float)kThetaMin) * ih;
            const int k = std::min(8, std::max(0, (int)std::floor(pos)));
            const float B = pos - k, A = 1.f - B;
            S = A * t.y[k] + B * t.y[k + 1] + (A * A * A - A) * t.m[k] + (B * B * B - B) * t.m[k + 1];
            dS = ((t.y[k + 1] - t.y[k]) + (1.f - 3.f * A * A) * t.m[k] + (3.f * B * B - 1.f) * t.m[k + 1]) * ih;
        }
        const float dE = a.kk * dS;
        const float uu = ux * ux + uy * uy + uz * uz, vv = vx * vx + vy * vy + vz * vz;
        const float c1 = -dE / (uu * nl), c3 = dE / (vv * nl);
        const float f1x = c1 * (uy * nz - uz * ny), f1y = c1 * (uz * nx - ux * nz), f1z = c1 * (ux * ny - uy * nx);
        const float f3x = c3 * (vy * nz - vz * ny), f3y = c3 * (vz * nx - vx * nz), f3z = c3 * (vx * ny - vy * nx);
        fx[a.i] += f1x; fy[a.i] += f1y; fz[a.i] += f1z;
        fx[a.k] += f3x; fy[a.k] += f3y; fz[a.k] += f3z;
        fx[a.j] -= f1x + f3x; fy[a.j] -= f1y + f3y; fz[a.j] -= f1z + f3z;
        if (energy) E[6] += a.kk * (S - t.emin);
    }
    // flexible-local dihedrals (Fourier series in cos/sin of phi)
    for (const Fld& d : s.fld) {
        const Fourier& t = s.fld_tab[d.table];
        const float Fx = X[d.i] - X[d.j], Fy = Y[d.i] - Y[d.j], Fz = Z[d.i] - Z[d.j];
        const float Gx = X[d.j] - X[d.k], Gy = Y[d.j] - Y[d.k], Gz = Z[d.j] - Z[d.k];
        const float Hx = X[d.l] - X[d.k], Hy = Y[d.l] - Y[d.k], Hz = Z[d.l] - Z[d.k];
        const float Ax = Fy * Gz - Fz * Gy, Ay = Fz * Gx - Fx * Gz, Az = Fx * Gy - Fy * Gx;
        const float Bx = Hy * Gz - Hz * Gy, By = Hz * Gx - Hx * Gz, Bz = Hx * Gy - Hy * Gx;
        const float AA = std::max(Ax * Ax + Ay * Ay + Az * Az, 1e-30f);
        const float BB = std::max(Bx * Bx + By * By + Bz * Bz, 1e-30f);
        const float Gl = std::sqrt(Gx * Gx + Gy * Gy + Gz * Gz);
        const float iab = 1.f / std::sqrt(AA * BB);
        const float c1 = (Ax * Bx + Ay * By + Az * Bz) * iab;
        const float s1 = -Gl * (Fx * Bx + Fy * By + Fz * Bz) * iab;
        const float c2 = c1 * c1 - s1 * s1, s2 = 2.f * s1 * c1;
        const float c3 = c1 * c2 - s1 * s2, s3 = s1 * c2 + c1 * s2;
        const float dE = d.kk * (-t.c[1] * s1 + t.c[2] * c1 - 2.f * t.c[3] * s2 + 2.f * t.c[4] * c2 -
                                 3.f * t.c[5] * s3 + 3.f * t.c[6] * c3);
        if (energy)
            E[7] += d.kk * (t.c[0] - t.emin + t.c[1] * c1 + t.c[2] * s1 + t.c[3] * c2 + t.c[4] * s2 +
                            t.c[5] * c3 + t.c[6] * s3);
        const float ga = Gl / AA, gb = Gl / BB;
        const float fg = (Fx * Gx + Fy * Gy + Fz * Gz) / (AA * Gl), hg = (Hx * Gx + Hy * Gy + Hz * Gz) / (BB * Gl);
        // f = -dE dphi/dx
        fx[d.i] += dE * ga * Ax; fy[d.i] += dE * ga * Ay; fz[d.i] += dE * ga * Az;
        fx[d.l] -= dE * gb * Bx; fy[d.l] -= dE * gb * By; fz[d.l] -= dE * gb * Bz;
        fx[d.j] -= dE * ((ga + fg) * Ax - hg * Bx);
        fy[d.j] -= dE * ((ga + fg) * Ay - hg * By);
        fz[d.j] -= dE * ((ga + fg) * Az - hg * Bz);
        fx[d.k] -= dE * (-fg * Ax + (hg - gb) * Bx);
        fy[d.k] -= dE * (-fg * Ay + (hg - gb) * By);
        fz[d.k] -= dE * (-fg * Az + (hg - gb) * Bz);
    }
    // pair terms over the half list
    const float tw13 = 1.2599210498948732f;  // 2^(1/3)
    for (int64_t i = 0; i < n; ++i) {
        const float xi = X[i], yi = Y[i], zi = Z[i];
        float ax = 0.f, ay = 0.f, az = 0.f;
        for (int32_t p = s.nb_start[i]; p < s.nb_start[i + 1]; ++p) {
            const int32_t j = s.nb_j[p];
            float dx = X[j] - xi, dy = Y[j] - yi, dz = Z[j] - zi;
            if (s.periodic) {
                dx = min_image(dx, bx, ibx);
                dy = min_image(dy, by, iby);
                dz = min_image(dz, bz, ibz);
            }
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 >= s.pair_rc2) continue;
            const uint8_t ex = s.nb_bits[p];
            const float ir2 = 1.f / r2;
            float sc = 0.f;  // F_i = -sc d
            if (s.exv && !(ex & 1) && r2 < s.exv_rc2) {
                const float S = s.rad[i] + s.rad[j];
                const float u = S * S * ir2, u3 = u * u * u, u6 = u3 * u3;
                sc += 12.f * s.exv_eps * u6 * ir2;
                if (energy) {
                    const float w = S * S * s.exv_corr, w3 = w * w * w;
                    E[0] += s.exv_eps * (u6 - w3 * w3);
                }
            }
            if (s.dh && !(ex & 2) && r2 < s.dh_rc2 && s.q[i] != 0.f && s.q[j] != 0.f) {
                const float r = std::sqrt(r2);
                const float e = std::exp(-r * s.dh_il);
                const float qq = s.q[i] * s.q[j] * s.dh_k;
                sc += qq * e * (s.dh_il + 1.f / r) * ir2;
                if (energy) E[1] += qq * (e / r - s.dh_corr);
            }
            if (s.ljr && !(ex & 4) && r2 < s.ljr_rc2) {
                const float sg = 0.5f * (s.ljr_sig[i] + s.ljr_sig[j]);
                if (r2 <= sg * sg * tw13) {
                    const float e = 0.5f * (s.ljr_eps[i] + s.ljr_eps[j]);
                    const float q2 = sg * sg * ir2, s6 = q2 * q2 * q2, s12 = s6 * s6;
                    sc += 24.f * e * (2.f * s12 - s6) * ir2;
                    if (energy) E[2] += e * (4.f * (s12 - s6) + 1.f);
                }
            }
            if (s.lja && !(ex & 8) && r2 < s.lja_rc2) {
                const float sg = 0.5f * (s.lja_sig[i] + s.lja_sig[j]);
                const float e = 0.5f * (s.lja_eps[i] + s.lja_eps[j]);
                float En, g;  // g = dE/dr / r
                if (r2 < sg * sg * tw13) {
                    En = -e;
                    g = 0.f;
                } else {
                    const float q2 = sg * sg * ir2, s6 = q2 * q2 * q2, s12 = s6 * s6;
                    En = 4.f * e * (s12 - s6);
                    g = -24.f * e * (2.f * s12 - s6) * ir2;
                }
                const float r = std::sqrt(r2);
                if (r > s.lja_rs) {
                    const float xx = (r - s.lja_rs) * s.lja_iw, x2 = xx * xx, x3 = x2 * xx;
                    const float sw = 1.f + x3 * (-10.f + xx * (15.f - 6.f * xx));
                    const float dsw = x2 * (-30.f + xx * (60.f - 30.f * xx)) * s.lja_iw;
                    g = g * sw + En * dsw / r;
                    En *= sw;
                }
                sc -= g;
                if (energy) E[3] += En;
            }
            ax -= sc * dx; ay -= sc * dy; az -= sc * dz;
            fx[j] += sc * dx; fy[j] += sc * dy; fz[j] += sc * dz;
        }
        fx[i] += ax; fy[i] += ay; fz[i] += az;
    }
    if (energy)
        for (int k = 0; k < 8; ++k) s.energy[k] = E[k];
}

bool needs_build(const CpuSystem& s) {
    const float lim = 0.25f * kSkin * kSkin;
    for (int64_t i = 0; i < s.n; ++i) {
        const float dx = s.x[i] - s.rx[i], dy = s.y[i] - s.ry[i], dz = s.z[i] - s.rz[i];
        if (dx * dx + dy * dy + dz * dz > lim) return true;
    }
    return false;
}

void advance(CpuSystem& s, int64_t steps) {
    for (int64_t k = 0; k < steps; ++k) {
        if (s.nb_start.empty() || needs_build(s)) build_list(s);
        forces(s, false);
        for (int64_t i = 0; i < s.n; ++i) {
            const float im = s.im[i];
            if (!(im > 0.f)) continue;
            float g[3];
            gaussian3f(s.seed, (uint32_t)i, s.step, g);
            const float sq = std::sqrt(im) * s.noise, fs = s.fscale * im;
            s.vx[i] = s.vscale * s.vx[i] + fs * s.fx[i] + sq * g[0];
            s.vy[i] = s.vscale * s.vy[i] + fs * s.fy[i] + sq * g[1];
            s.vz[i] = s.vscale * s.vz[i] + fs * s.fz[i] + sq * g[2];
            s.x[i] += s.vx[i] * s.dt;
            s.y[i] += s.vy[i] * s.dt;
            s.z[i] += s.vz[i] * s.dt;
        }
        ++s.step;
    }
}

}  // namespace

extern "C" {

// Set-up of one system (untimed): derived constants, tables, exclusions.
// Returns 0, or 6 if the system uses a feature this restatement refuses.
int cpu_prepare(const OracleSystem* o, const double* vel, const double* mass, double T, double gamma,
                double dt, uint32_t seed, void** out) {
    *out = nullptr;
    if (o->grp || o->ljr_side || o->lja_side || o->ljr_geometric || o->n_cgo || o->n_gb || o->n_gd ||
        o->ign_molecule[0] || o->ign_molecule[1] || o->ign_molecule[2] || o->ign_molecule[3])
        return 6;
    auto* s = new CpuSystem();
    const int64_t n = o->n;
    s->n = n;
    s->periodic = o->periodic != 0;
    s->bond_pbc = o->bond_periodic != 0 && s->periodic;
    s->go_pbc = o->go_periodic != 0 && s->periodic;
    for (int c = 0; c < 3; ++c) s->box[c] = (float)o->box[c];
    s->x.resize(n); s->y.resize(n); s->z.resize(n);
    s->vx.assign(n, 0.f); s->vy.assign(n, 0.f); s->vz.assign(n, 0.f);
    s->fx.assign(n, 0.f); s->fy.assign(n, 0.f); s->fz.assign(n, 0.f);
    s->im.resize(n);
    for (int64_t i = 0; i < n; ++i) {
        s->x[i] = (float)o->pos[3 * i];
        s->y[i] = (float)o->pos[3 * i + 1];
        s->z[i] = (float)o->pos[3 * i + 2];
        if (vel) {
            s->vx[i] = (float)vel[3 * i];
            s->vy[i] = (float)vel[3 * i + 1];
            s->vz[i] = (float)vel[3 * i + 2];
        }
        s->im[i] = mass[i] > 0 ? (float)(1.0 / mass[i]) : 0.f;
    }
    for (int64_t b = 0; b < o->n_bonds; ++b)
        s->bonds.push_back({(int32_t)o->bond_idx[2 * b], (int32_t)o->bond_idx[2 * b + 1], (float)o->bond_v0[b],
                            (float)o->bond_k[b]});
    for (int64_t b = 0; b < o->n_go; ++b)
        s->go.push_back({(int32_t)o->go_idx[2 * b], (int32_t)o->go_idx[2 * b + 1], (float)o->go_k[b],
                         (float)o->go_r0[b]});
    const double h = (kThetaMax - kThetaMin) / 9.0;
    int fla_map[20];
    std::fill(fla_map, fla_map + 20, -1);
    for (int64_t a = 0; a < o->n_fla; ++a) {
        const int aa = o->fla_aa[a];
        if (fla_map[aa] < 0) {
            double M[10];
            oracle_natural_spline(kFlaY[aa], h, M);
            Table t;
            for (int k = 0; k < 10; ++k) {
                t.y[k] = (float)kFlaY[aa][k];
                t.m[k] = (float)(M[k] * h * h / 6.0);
            }
            t.emin = (float)oracle_fla_min_energy(aa);
            fla_map[aa] = (int)s->fla_tab.size();
            s->fla_tab.push_back(t);
        }
        s->fla.push_back({(int32_t)o->fla_idx[3 * a], (int32_t)o->fla_idx[3 * a + 1], (int32_t)o->fla_idx[3 * a + 2],
                          (float)o->fla_k[a], fla_map[aa]});
    }
    int fld_map[23];
    std::fill(fld_map, fld_map + 23, -1);
    for (int64_t q = 0; q < o->n_fld; ++q) {
        int32_t cls[4];
        const int nc = oracle_fld_classes(o->fld_aa1[q], o->fld_aa2[q], cls, 4);
        for (int c = 0; c < nc; ++c) {
            if (fld_map[cls[c]] < 0) {
                Fourier f;
                for (int k = 0; k < 7; ++k) f.c[k] = (float)kFld[cls[c]].c[k];
                f.emin = (float)oracle_fld_min_energy(cls[c]);
                fld_map[cls[c]] = (int)s->fld_tab.size();
                s->fld_tab.push_back(f);
            }
            s->fld.push_back({(int32_t)o->fld_idx[4 * q], (int32_t)o->fld_idx[4 * q + 1],
                              (int32_t)o->fld_idx[4 * q + 2], (int32_t)o->fld_idx[4 * q + 3], (float)o->fld_k[q],
                              fld_map[cls[c]]});
        }
    }
    // pair terms: cutoffs from the generators' ratios, as the oracle derives them
    double rcmax = 0;
    auto present = [](const double* v, int64_t n) {
        std::vector<float> out(n);
        for (int64_t i = 0; i < n; ++i) out[i] = std::isnan(v[i]) ? 0.f : (float)v[i];
        return out;
    };
    auto all_present = [](const double* v, int64_t n) {
        for (int64_t i = 0; i < n; ++i)
            if (std::isnan(v[i])) return false;
        return true;
    };
    if (o->exv_on) {
        if (!all_present(o->exv_radius, n)) { delete s; return 6; }
        double t2[2];
        oracle_top_two(o->exv_radius, n, 1, t2);
        const double rc = (t2[0] + t2[1]) * o->exv_ratio;
        s->exv = true;
        s->exv_eps = (float)o->exv_eps;
        s->exv_rc2 = (float)(rc * rc);
        s->exv_corr = (float)(1.0 / (rc * rc));
        s->rad = present(o->exv_radius, n);
        rcmax = std::max(rcmax, rc);
    }
    if (o->dh_on) {
        double p[5];
        oracle_dh_params(o->dh_I, o->dh_T, o->dh_ratio, p);
        s->dh = true;
        s->dh_k = (float)p[0];
        s->dh_il = (float)(1.0 / p[1]);
        s->dh_rc2 = (float)(p[2] * p[2]);
        s->dh_corr = (float)p[3];
        s->q = present(o->dh_q, n);  // absent = no charge
        rcmax = std::max(rcmax, p[2]);
    }
    if (o->ljr_on) {
        if (!all_present(o->ljr_sigma, n)) { delete s; return 6; }
        double t2[2];
        oracle_top_two(o->ljr_sigma, n, 0, t2);
        const double rc = (t2[0] + t2[1]) * 0.5 * o->ljr_ratio;
        s->ljr = true;
        s->ljr_rc2 = (float)(rc * rc);
        s->ljr_eps = present(o->ljr_eps, n);
        s->ljr_sig = present(o->ljr_sigma, n);
        rcmax = std::max(rcmax, rc);
    }
    if (o->lja_on) {
        if (!all_present(o->lja_sigma, n)) { delete s; return 6; }
        double t2[2];
        oracle_top_two(o->lja_sigma, n, 0, t2);
        const double rc = (t2[0] + t2[1]) * 0.5 * o->lja_ratio;
        s->lja = true;
        s->lja_rc2 = (float)(rc * rc);
        s->lja_rs = (float)(0.9 * rc);
        s->lja_iw = (float)(1.0 / (rc - 0.9 * rc));
        s->lja_eps = present(o->lja_eps, n);
        s->lja_sig = present(o->lja_sigma, n);
        rcmax = std::max(rcmax, rc);
    }
    s->pair_rc2 = std::max(std::max(s->exv_rc2, s->dh_rc2), std::max(s->ljr_rc2, s->lja_rc2));
    s->list_rc = (float)rcmax + kSkin;
    s->list_rc2 = s->list_rc * s->list_rc;
    // exclusions per term, merged into per-pair bits
    std::vector<std::vector<std::pair<int32_t, uint8_t>>> ex(n);
    const int ign[4][2] = {{o->exv_ign_bond, o->exv_ign_contact}, {o->dh_ign_bond, o->dh_ign_contact},
                           {o->ljr_ign_bond, o->ljr_ign_contact}, {o->lja_ign_bond, o->lja_ign_contact}};
    const int on[4] = {o->exv_on, o->dh_on, o->ljr_on, o->lja_on};
    for (int t = 0; t < 4; ++t) {
        if (!on[t]) continue;
        int64_t cnt = 0;
        oracle_ignore_within(n, o->n_bonds, o->bond_idx, o->n_go, o->go_idx, ign[t][0], ign[t][1], nullptr, 0, &cnt);
        std::vector<int64_t> pairs(2 * std::max<int64_t>(cnt, 1));
        oracle_ignore_within(n, o->n_bonds, o->bond_idx, o->n_go, o->go_idx, ign[t][0], ign[t][1], pairs.data(),
                             cnt, &cnt);
        for (int64_t k = 0; k < cnt; ++k) ex[pairs[2 * k]].emplace_back((int32_t)pairs[2 * k + 1], (uint8_t)(1 << t));
    }
    s->ex_start.assign(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) {
        auto& v = ex[i];
        std::sort(v.begin(), v.end());
        for (std::size_t k = 0; k < v.size(); ++k) {
            if (k > 0 && v[k].first == v[k - 1].first) {
                s->ex_bits.back() |= v[k].second;  // the same pair excluded for another term
            } else {
                s->ex_j.push_back(v[k].first);
                s->ex_bits.push_back(v[k].second);
            }
        }
        s->ex_start[i + 1] = (int32_t)s->ex_j.size();
    }
    const double a = std::exp(-gamma * dt);
    s->vscale = (float)a;
    s->fscale = (float)(gamma == 0 ? dt : (1 - a) / gamma);
    s->noise = (float)std::sqrt(kBoltz * T * (1 - a * a));
    s->dt = (float)dt;
    s->seed = seed;
    *out = s;
    return 0;
}

// `steps` Langevin steps of every system, OpenMP over systems (largest
// first, dynamic), on `threads` threads (0: all).
int cpu_run_many(void** systems, int64_t count, int64_t steps, int threads) {
    std::vector<int64_t> order(count);
    for (int64_t k = 0; k < count; ++k) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
        return static_cast<CpuSystem*>(systems[a])->n > static_cast<CpuSystem*>(systems[b])->n;
    });
    const int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int64_t k = 0; k < count; ++k) advance(*static_cast<CpuSystem*>(systems[order[k]]), steps);
    return 0;
}

int cpu_max_threads(void) { return omp_get_max_threads(); }

// Forces and the energies of the EXV, DH, LJR, LJA, HB, GO, FLA, FLD slots
// at the current positions (FP32 arithmetic, reported in FP64).
int cpu_evaluate(void* h, double* f, double* e8) {
    CpuSystem& s = *static_cast<CpuSystem*>(h);
    build_list(s);
    forces(s, true);
    for (int64_t i = 0; i < s.n; ++i) {
        f[3 * i] = s.fx[i];
        f[3 * i + 1] = s.fy[i];
        f[3 * i + 2] = s.fz[i];
    }
    for (int k = 0; k < 8; ++k) e8[k] = s.energy[k];
    return 0;
}

int cpu_get_positions(void* h, double* x) {
    const CpuSystem& s = *static_cast<CpuSystem*>(h);
    for (int64_t i = 0; i < s.n; ++i) {
        x[3 * i] = s.x[i];
        x[3 * i + 1] = s.y[i];
        x[3 * i + 2] = s.z[i];
    }
    return 0;
}

void cpu_free(void* h) { delete static_cast<CpuSystem*>(h); }

}  // extern "C"
