// capi.cpp - the extern "C" boundary (include/ocm.h).  Converts C arrays
// into the host mirrors of the reference's classes and every C++ exception
// into a status code plus a thread-local message.
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <string>

#include "../../include/ocm.h"
#include "batch_engine.hpp"
#include "engine.hpp"
#include "host_system.hpp"

struct ocm_topology {
    ocm::Topology t;
    explicit ocm_topology(std::size_t n) : t(n) {}
};
struct ocm_system {
    ocm::SystemGenerator g;
    explicit ocm_system(std::vector<double> m) : g(std::move(m)) {}
};
struct ocm_context {
    std::unique_ptr<ocm::PlainContext> c;
};
struct ocm_batch {
    std::unique_ptr<ocm::BatchEngine> b;
};

namespace {

thread_local std::string g_error;

template <class F>
int guard(F&& f) {
    try {
        f();
        return OCM_OK;
    } catch (const ocm::Error& e) {
        g_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_error = "[error] host allocation failed";
        return OCM_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        g_error = e.what();
        return OCM_ERR_INVALID_ARGUMENT;
    } catch (...) {
        g_error = "[error] unknown exception";
        return OCM_ERR_INVALID_ARGUMENT;
    }
}

void need(const void* p, const char* what) {
    if (!p) throw ocm::Error(OCM_ERR_INVALID_ARGUMENT, std::string("[error] null pointer: ") + what);
}

int write_pairs(const std::vector<std::pair<std::size_t, std::size_t>>& v, int64_t* out,
                int64_t cap, int64_t* n_out) {
    *n_out = (int64_t)v.size();
    if ((int64_t)v.size() > cap) {
        g_error = "[error] output capacity too small";
        return OCM_ERR_INVALID_ARGUMENT;
    }
    for (std::size_t k = 0; k < v.size(); ++k) {
        out[2 * k] = (int64_t)v[k].first;
        out[2 * k + 1] = (int64_t)v[k].second;
    }
    return OCM_OK;
}

ocm::PairGeneratorCommon common_args(const ocm_system* sys, int64_t n_ignore,
                                     const int64_t* ignore, int use_periodic, int64_t n_ig,
                                     const int32_t* igp, const int32_t* group_vec) {
    ocm::PairGeneratorCommon c;
    if (n_ignore < 0 || n_ig < 0) throw ocm::Error(1, "[error] negative count");
    if (n_ignore) need(ignore, "ignore_pairs");
    for (int64_t k = 0; k < n_ignore; ++k) c.ignore_list.emplace_back(ignore[2 * k], ignore[2 * k + 1]);
    c.use_periodic = use_periodic != 0;
    if (n_ig) {
        need(igp, "ignore_group_pairs");
        need(group_vec, "group_vec");
        for (int64_t k = 0; k < n_ig; ++k) c.ignore_group_pairs.emplace_back(igp[2 * k], igp[2 * k + 1]);
        const int64_t n = (int64_t)sys->g.desc().masses.size();
        c.group_vec.assign(group_vec, group_vec + n);
    }
    return c;
}

std::vector<double> copy_vec(const double* p, int64_t n, const char* what) {
    if (n) need(p, what);
    return std::vector<double>(p, p + n);
}

}  // namespace

extern "C" {

const char* ocm_last_error(void) { return g_error.c_str(); }
int ocm_abi_version(void) { return OCM_ABI_VERSION; }
int ocm_device_count(void) {
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return c;
}

int ocm_fla_table(const char* aa, double* y, double* d2y) {
    return guard([&] {
        need(aa, "aa_name");
        const auto* t = ocm::fla_spline_table(aa);
        const auto* d = ocm::fla_second_derivative_table(aa);
        if (!t || !d) throw ocm::Error(1, std::string("[error] unknown amino acid ") + aa);
        if (y) std::memcpy(y, t->data(), 10 * sizeof(double));
        if (d2y) std::memcpy(d2y, d->data(), 10 * sizeof(double));
    });
}
int ocm_fld_table(const char* key, double* f) {
    return guard([&] {
        need(key, "key");
        const auto* t = ocm::fld_fourier_table(key);
        if (!t) throw ocm::Error(1, std::string("[error] unknown dihedral class ") + key);
        if (f) std::memcpy(f, t->data(), 7 * sizeof(double));
    });
}
int ocm_fld_table_key(int idx, char* buf, int64_t cap) {
    return guard([&] {
        const auto& k = ocm::fld_table_keys();
        if (idx < 0 || idx >= (int)k.size()) throw ocm::Error(1, "[error] table index out of range");
        need(buf, "buf");
        if ((int64_t)k[idx].size() + 1 > cap) throw ocm::Error(1, "[error] buffer too small");
        std::memcpy(buf, k[idx].c_str(), k[idx].size() + 1);
    });
}

// ---------------- topology ----------------
int ocm_topology_create(int64_t n, ocm_topology** out) {
    return guard([&] {
        need(out, "out");
        if (n < 0) throw ocm::Error(1, "[error] negative size");
        *out = new ocm_topology((std::size_t)n);
    });
}
void ocm_topology_destroy(ocm_topology* t) { delete t; }
int ocm_topology_add_edges(ocm_topology* t, int64_t n, const int64_t* pairs, const char* type) {
    return guard([&] {
        need(t, "topology");
        need(type, "edge_type");
        if (n) need(pairs, "pairs");
        std::vector<std::pair<std::size_t, std::size_t>> e;
        for (int64_t k = 0; k < n; ++k) {
            if (pairs[2 * k] < 0 || pairs[2 * k + 1] < 0) throw ocm::Error(1, "[error] negative index");
            e.emplace_back((std::size_t)pairs[2 * k], (std::size_t)pairs[2 * k + 1]);
        }
        t->t.add_edges(e, type);
    });
}
int ocm_topology_make_molecule(ocm_topology* t, const char* type) {
    return guard([&] {
        need(t, "topology");
        need(type, "edge_type");
        t->t.make_molecule(type);
    });
}
int ocm_topology_ignore_list_within_edge(const ocm_topology* t, int64_t dist, const char* type,
                                         int64_t* out, int64_t cap, int64_t* n_out) {
    int rc = OCM_OK;
    const int g = guard([&] {
        need(t, "topology");
        need(type, "edge_type");
        need(n_out, "n_out");
        if (dist < 0) throw ocm::Error(1, "[error] negative distance");
        rc = write_pairs(t->t.ignore_list_within_edge((std::size_t)dist, type), out, cap, n_out);
    });
    return g ? g : rc;
}
int ocm_topology_ignore_list_within_molecule(const ocm_topology* t, int64_t* out, int64_t cap,
                                             int64_t* n_out) {
    int rc = OCM_OK;
    const int g = guard([&] {
        need(t, "topology");
        need(n_out, "n_out");
        rc = write_pairs(t->t.ignore_list_within_molecule(), out, cap, n_out);
    });
    return g ? g : rc;
}

// ---------------- system ----------------
int ocm_system_create(int64_t n, const double* masses, ocm_system** out) {
    return guard([&] {
        need(out, "out");
        if (n < 0) throw ocm::Error(1, "[error] negative size");
        *out = new ocm_system(copy_vec(masses, n, "masses"));
    });
}
void ocm_system_destroy(ocm_system* s) { delete s; }
int ocm_system_set_pbc(ocm_system* s, double x, double y, double z) {
    return guard([&] {
        need(s, "system");
        s->g.set_pbc(x, y, z);
    });
}
int64_t ocm_system_num_particles(const ocm_system* s) {
    return s ? (int64_t)s->g.desc().masses.size() : -1;
}
int ocm_system_num_groups(const ocm_system* s) {
    return s ? (int)s->g.desc().group_names.size() : -1;
}
int ocm_system_group_name(const ocm_system* s, int g, char* buf, int64_t cap) {
    return guard([&] {
        need(s, "system");
        need(buf, "buf");
        const auto& names = s->g.desc().group_names;
        if (g < 0 || g >= (int)names.size()) throw ocm::Error(1, "[error] group out of range");
        if ((int64_t)names[g].size() + 1 > cap) throw ocm::Error(1, "[error] buffer too small");
        std::memcpy(buf, names[g].c_str(), names[g].size() + 1);
    });
}
int ocm_system_describe(const ocm_system* s, char* buf, int64_t cap, int64_t* needed) {
    return guard([&] {
        need(s, "system");
        const std::string j = s->g.describe_json();
        if (needed) *needed = (int64_t)j.size() + 1;
        if (buf) {
            if ((int64_t)j.size() + 1 > cap) throw ocm::Error(1, "[error] buffer too small");
            std::memcpy(buf, j.c_str(), j.size() + 1);
        }
    });
}

static std::vector<std::pair<int64_t, int64_t>> pairs_of(const int64_t* p, int64_t n) {
    std::vector<std::pair<int64_t, int64_t>> v;
    if (n < 0) throw ocm::Error(1, "[error] negative count");
    if (n) need(p, "indices");
    for (int64_t k = 0; k < n; ++k) {
        if (p[2 * k] < 0 || p[2 * k + 1] < 0) throw ocm::Error(1, "[error] negative index");
        v.emplace_back(p[2 * k], p[2 * k + 1]);
    }
    return v;
}

int ocm_add_harmonic_bond(ocm_system* s, int64_t n, const int64_t* idx, const double* v0s,
                          const double* ks, int use_periodic, int* group_out) {
    return guard([&] {
        need(s, "system");
        auto g = std::make_unique<ocm::HarmonicBondForceFieldGenerator>(
            pairs_of(idx, n), copy_vec(v0s, n, "v0s"), copy_vec(ks, n, "ks"), use_periodic != 0);
        const int grp = s->g.add_ff_generator(std::move(g));
        if (group_out) *group_out = grp;
    });
}
int ocm_add_go_contact(ocm_system* s, int64_t n, const int64_t* idx, const double* ks,
                       const double* r0s, int use_periodic, int* group_out) {
    return guard([&] {
        need(s, "system");
        auto g = std::make_unique<ocm::GoContactForceFieldGenerator>(
            pairs_of(idx, n), copy_vec(ks, n, "ks"), copy_vec(r0s, n, "r0s"), use_periodic != 0);
        const int grp = s->g.add_ff_generator(std::move(g));
        if (group_out) *group_out = grp;
    });
}
int ocm_add_gaussian_bond(ocm_system* s, int64_t n, const int64_t* idx, const double* ks,
                          const double* v0s, const double* sigmas, int use_periodic, int* group_out) {
    return guard([&] {
        need(s, "system");
        auto g = std::make_unique<ocm::GaussianBondForceFieldGenerator>(
            pairs_of(idx, n), copy_vec(ks, n, "ks"), copy_vec(v0s, n, "v0s"),
            copy_vec(sigmas, n, "sigmas"), use_periodic != 0);
        const int grp = s->g.add_ff_generator(std::move(g));
        if (group_out) *group_out = grp;
    });
}
int ocm_add_gaussian_dihedral(ocm_system* s, int64_t n, const int64_t* idx, const double* ks,
                              const double* theta0s, const double* sigmas, int use_periodic,
                              int* group_out) {
    return guard([&] {
        need(s, "system");
        if (n < 0) throw ocm::Error(1, "[error] negative count");
        if (n) need(idx, "indices");
        std::vector<std::array<int64_t, 4>> v;
        for (int64_t k = 0; k < n; ++k) {
            for (int c = 0; c < 4; ++c)
                if (idx[4 * k + c] < 0) throw ocm::Error(1, "[error] negative index");
            v.push_back({idx[4 * k], idx[4 * k + 1], idx[4 * k + 2], idx[4 * k + 3]});
        }
        auto g = std::make_unique<ocm::GaussianDihedralForceFieldGenerator>(
            std::move(v), copy_vec(ks, n, "ks"), copy_vec(theta0s, n, "theta0s"),
            copy_vec(sigmas, n, "sigmas"), use_periodic != 0);
        const int grp = s->g.add_ff_generator(std::move(g));
        if (group_out) *group_out = grp;
    });
}
int ocm_add_flexible_local_angle(ocm_system* s, int64_t n, const int64_t* idx, const double* ks,
                                 const double* table, const char* aa, int use_periodic,
                                 int* group_out) {
    return guard([&] {
        need(s, "system");
        need(table, "spline_table");
        need(aa, "aa_name");
        if (n < 0) throw ocm::Error(1, "[error] negative count");
        if (n) need(idx, "indices");
        std::vector<std::array<int64_t, 3>> v;
        for (int64_t k = 0; k < n; ++k) {
            for (int c = 0; c < 3; ++c)
                if (idx[3 * k + c] < 0) throw ocm::Error(1, "[error] negative index");
            v.push_back({idx[3 * k], idx[3 * k + 1], idx[3 * k + 2]});
        }
        std::array<double, 10> t;
        std::memcpy(t.data(), table, sizeof(t));
        auto g = std::make_unique<ocm::FlexibleLocalAngleForceFieldGenerator>(
            std::move(v), copy_vec(ks, n, "ks"), t, aa, use_periodic != 0);
        const int grp = s->g.add_ff_generator(std::move(g));
        if (group_out) *group_out = grp;
    });
}
int ocm_add_flexible_local_dihedral(ocm_system* s, int64_t n, const int64_t* idx, const double* ks,
                                    const double* table, const char* name, int use_periodic,
                                    int* group_out) {
    return guard([&] {
        need(s, "system");
        need(table, "fourier_table");
        need(name, "aa_pair_name");
        if (n < 0) throw ocm::Error(1, "[error] negative count");
        if (n) need(idx, "indices");
        std::vector<std::array<int64_t, 4>> v;
        for (int64_t k = 0; k < n; ++k) {
            for (int c = 0; c < 4; ++c)
                if (idx[4 * k + c] < 0) throw ocm::Error(1, "[error] negative index");
            v.push_back({idx[4 * k], idx[4 * k + 1], idx[4 * k + 2], idx[4 * k + 3]});
        }
        std::array<double, 7> t;
        std::memcpy(t.data(), table, sizeof(t));
        auto g = std::make_unique<ocm::FlexibleLocalDihedralForceFieldGenerator>(
            std::move(v), copy_vec(ks, n, "ks"), t, name, use_periodic != 0);
        const int grp = s->g.add_ff_generator(std::move(g));
        if (group_out) *group_out = grp;
    });
}
int ocm_add_excluded_volume(ocm_system* s, double eps, double ratio, const double* radii,
                            int64_t n_ignore, const int64_t* ignore, int use_periodic,
                            int64_t n_ig, const int32_t* igp, const int32_t* gv, int* group_out) {
    return guard([&] {
        need(s, "system");
        const int64_t n = (int64_t)s->g.desc().masses.size();
        auto g = std::make_unique<ocm::ExcludedVolumeForceFieldGenerator>(
            eps, ratio, copy_vec(radii, n, "radii"),
            common_args(s, n_ignore, ignore, use_periodic, n_ig, igp, gv));
        const int grp = s->g.add_ff_generator(std::move(g));
        if (group_out) *group_out = grp;
    });
}
int ocm_add_debye_huckel(ocm_system* s, double ionic, double T, double ratio, const double* q,
                         int64_t n_ignore, const int64_t* ignore, int use_periodic, int64_t n_ig,
                         const int32_t* igp, const int32_t* gv, int* group_out) {
    return guard([&] {
        need(s, "system");
        const int64_t n = (int64_t)s->g.desc().masses.size();
        auto g = std::make_unique<ocm::DebyeHuckelForceFieldGenerator>(
            ionic, T, ratio, copy_vec(q, n, "charges"),
            common_args(s, n_ignore, ignore, use_periodic, n_ig, igp, gv));
        const int grp = s->g.add_ff_generator(std::move(g));
        if (group_out) *group_out = grp;
    });
}
static int add_lj(bool attr, ocm_system* s, double ratio, const double* eps, const double* sig,
                  int64_t n_ignore, const int64_t* ignore, int use_periodic, int64_t n_ig,
                  const int32_t* igp, const int32_t* gv, int* group_out) {
    return guard([&] {
        need(s, "system");
        const int64_t n = (int64_t)s->g.desc().masses.size();
        auto g = std::make_unique<ocm::LennardJonesForceFieldGenerator>(
            attr, ratio, copy_vec(eps, n, "epsilons"), copy_vec(sig, n, "sigmas"),
            common_args(s, n_ignore, ignore, use_periodic, n_ig, igp, gv));
        const int grp = s->g.add_ff_generator(std::move(g));
        if (group_out) *group_out = grp;
    });
}
int ocm_add_lennard_jones_repulsive(ocm_system* s, double ratio, const double* eps,
                                    const double* sig, int64_t n_ignore, const int64_t* ignore,
                                    int use_periodic, int64_t n_ig, const int32_t* igp,
                                    const int32_t* gv, int* group_out) {
    return add_lj(false, s, ratio, eps, sig, n_ignore, ignore, use_periodic, n_ig, igp, gv, group_out);
}
int ocm_add_lennard_jones_attractive(ocm_system* s, double ratio, const double* eps,
                                     const double* sig, int64_t n_ignore, const int64_t* ignore,
                                     int use_periodic, int64_t n_ig, const int32_t* igp,
                                     const int32_t* gv, int* group_out) {
    return add_lj(true, s, ratio, eps, sig, n_ignore, ignore, use_periodic, n_ig, igp, gv, group_out);
}

int ocm_add_weeks_chandler_andersen(ocm_system* s, const double* sig, const double* eps, int64_t n_ignore,
                                    const int64_t* ignore, int use_periodic, int64_t n_ig,
                                    const int32_t* igp, const int32_t* gv, int* group_out) {
    return guard([&] {
        need(s, "system");
        const int64_t n = (int64_t)s->g.desc().masses.size();
        auto g = std::make_unique<ocm::WeeksChandlerAndersenForceFieldGenerator>(
            copy_vec(sig, n, "sigmas"), copy_vec(eps, n, "epsilons"),
            common_args(s, n_ignore, ignore, use_periodic, n_ig, igp, gv));
        const int grp = s->g.add_ff_generator(std::move(g));
        if (group_out) *group_out = grp;
    });
}

static std::vector<int64_t> index_list(int64_t n, const int64_t* v, const char* what) {
    if (n < 0) throw ocm::Error(1, "[error] negative count");
    if (n) need(v, what);
    return std::vector<int64_t>(v, v + n);
}

static int add_uniform(bool attr, ocm_system* s, double eps, double sigma, double ratio, int64_t n_former,
                       const int64_t* former, int64_t n_latter, const int64_t* latter, int64_t n_ignore,
                       const int64_t* ignore, int use_periodic, int64_t n_ig, const int32_t* igp,
                       const int32_t* gv, int* group_out) {
    return guard([&] {
        need(s, "system");
        const int64_t n = (int64_t)s->g.desc().masses.size();
        auto g = std::make_unique<ocm::UniformPairForceFieldGenerator>(
            attr, n, eps, sigma, ratio, index_list(n_former, former, "former"),
            index_list(n_latter, latter, "latter"),
            common_args(s, n_ignore, ignore, use_periodic, n_ig, igp, gv));
        const int grp = s->g.add_ff_generator(std::move(g));
        if (group_out) *group_out = grp;
    });
}
int ocm_add_uniform_weeks_chandler_andersen(ocm_system* s, double eps, double sigma, int64_t n_former,
                                            const int64_t* former, int64_t n_latter, const int64_t* latter,
                                            int64_t n_ignore, const int64_t* ignore, int use_periodic,
                                            int64_t n_ig, const int32_t* igp, const int32_t* gv,
                                            int* group_out) {
    return add_uniform(false, s, eps, sigma, 0.0, n_former, former, n_latter, latter, n_ignore, ignore,
                       use_periodic, n_ig, igp, gv, group_out);
}
int ocm_add_uniform_lennard_jones_attractive(ocm_system* s, double eps, double sigma, double cutoff_ratio,
                                             int64_t n_former, const int64_t* former, int64_t n_latter,
                                             const int64_t* latter, int64_t n_ignore, const int64_t* ignore,
                                             int use_periodic, int64_t n_ig, const int32_t* igp,
                                             const int32_t* gv, int* group_out) {
    return add_uniform(true, s, eps, sigma, cutoff_ratio, n_former, former, n_latter, latter, n_ignore,
                       ignore, use_periodic, n_ig, igp, gv, group_out);
}

int ocm_add_capped_go_contact(ocm_system* s, int64_t n, const int64_t* idx, const double* ks,
                              const double* r0s, double capping_ratio, int use_periodic, int* group_out) {
    return guard([&] {
        need(s, "system");
        auto g = std::make_unique<ocm::CappedGoContactForceFieldGenerator>(
            pairs_of(idx, n), copy_vec(ks, n, "ks"), copy_vec(r0s, n, "r0s"), capping_ratio,
            use_periodic != 0);
        const int grp = s->g.add_ff_generator(std::move(g));
        if (group_out) *group_out = grp;
    });
}

// ---------------- plain context ----------------

int ocm_context_create(const ocm_system* s, double T, double friction, double dt, int32_t seed,
                       int device, ocm_context** out) {
    return guard([&] {
        need(s, "system");
        need(out, "out");
        auto c = std::make_unique<ocm_context>();
        c->c = std::make_unique<ocm::PlainContext>(s->g.desc(), T, friction, dt, seed, device);
        *out = c.release();
    });
}
void ocm_context_destroy(ocm_context* c) { delete c; }

#define CTX_CALL(body)                 \
    return guard([&] {                 \
        need(ctx, "context");          \
        body;                          \
    })

int ocm_context_set_positions(ocm_context* ctx, const double* xyz) {
    CTX_CALL(need(xyz, "xyz"); ctx->c->set_positions(xyz));
}
int ocm_context_get_positions(ocm_context* ctx, double* xyz) {
    CTX_CALL(need(xyz, "xyz"); ctx->c->get_positions(xyz));
}
int ocm_context_set_velocities(ocm_context* ctx, const double* v) {
    CTX_CALL(need(v, "v"); ctx->c->set_velocities(v));
}
int ocm_context_get_velocities(ocm_context* ctx, double* v) {
    CTX_CALL(need(v, "v"); ctx->c->get_velocities(v));
}
int ocm_context_set_velocities_to_temperature(ocm_context* ctx, double T, int32_t seed) {
    CTX_CALL(ctx->c->set_velocities_to_temperature(T, seed));
}
int ocm_context_get_state(ocm_context* ctx, uint32_t groups, double* forces, double* energy) {
    CTX_CALL(ctx->c->get_state(groups, forces, energy));
}
int ocm_context_get_group_energies(ocm_context* ctx, double* e) {
    CTX_CALL(need(e, "energies"); ctx->c->group_energies(e));
}
int ocm_context_get_kinetic_energy(ocm_context* ctx, double* ke) {
    CTX_CALL(need(ke, "ke"); *ke = ctx->c->kinetic_energy());
}
int ocm_context_step(ocm_context* ctx, int64_t steps) { CTX_CALL(ctx->c->step(steps)); }
int ocm_context_minimize(ocm_context* ctx, double tolerance, int64_t max_iterations, int64_t* iterations_out) {
    CTX_CALL(const int64_t it = ctx->c->minimize(tolerance, max_iterations);
             if (iterations_out) *iterations_out = it);
}
int ocm_context_set_engine(ocm_context* ctx, int32_t mode) { CTX_CALL(ctx->c->set_engine(mode)); }
int ocm_context_minimize_report(ocm_context* ctx, int32_t* reason, double* rms_force) {
    CTX_CALL(need(reason, "reason"); const auto& c = *ctx->c;
             if (c.min_reason < 0) throw ocm::Error(5, "[error] no minimisation has run on this context");
             *reason = c.min_reason; if (rms_force) *rms_force = c.min_rms);
}
int ocm_context_get_stats(ocm_context* ctx, ocm_context_stats* out) {
    CTX_CALL(need(out, "out"); const auto& c = *ctx->c; out->steps_done = c.steps_done;
             out->list_builds = c.list_builds; out->tiles = c.tiles_last;
             out->masked_tiles = c.masked_last; out->rebuild_interval = c.rebuild_interval;
             out->reordered = c.reorder ? 1 : 0; out->skin = c.skin;
             out->max_cutoff = c.cs.max_cutoff; out->tile_cutoff = c.tile_cutoff();
             out->charged_pairs = c.charged_pairs(); out->charged_split = c.charged_split() ? 1 : 0;
             out->one_system = c.last_step_one_system() ? 1 : 0);
}
int ocm_context_set_list_options(ocm_context* ctx, int32_t interval, double skin) {
    CTX_CALL(ctx->c->set_list_options(interval, skin));
}
int ocm_context_list_pairs(ocm_context* ctx, int64_t* out, int64_t cap, int64_t* n_out) {
    CTX_CALL(need(out, "out"); need(n_out, "n_out"); ctx->c->list_pairs(out, cap, n_out));
}
int ocm_context_cluster_order(ocm_context* ctx, int64_t* order, int64_t cap, int64_t* n_out) {
    CTX_CALL(need(order, "order"); need(n_out, "n_out"); ctx->c->cluster_order(order, cap, n_out));
}

// ---------------- batch ----------------
int ocm_batch_create(int device, int64_t max_systems, int64_t max_total_beads,
                     int32_t max_beads_per_system, ocm_batch** out) {
    return guard([&] {
        need(out, "out");
        auto b = std::make_unique<ocm_batch>();
        b->b = std::make_unique<ocm::BatchEngine>(device, max_systems, max_total_beads,
                                                   max_beads_per_system);
        *out = b.release();
    });
}
void ocm_batch_destroy(ocm_batch* b) { delete b; }
int64_t ocm_batch_footprint(const ocm_system* s) {
    if (!s) return -1;
    try {
        return ocm::BatchEngine::footprint(s->g.desc());
    } catch (const std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

#define BATCH_CALL(body)               \
    return guard([&] {                 \
        need(batch, "batch");          \
        body;                          \
    })

int ocm_batch_admit(ocm_batch* batch, const ocm_system* s, const double* pos, const double* vel,
                    double T, double friction, double dt, int32_t seed, int64_t n_steps,
                    int64_t* slot_out) {
    BATCH_CALL(need(s, "system"); need(pos, "positions"); need(slot_out, "slot_out");
               *slot_out = batch->b->admit(s->g.desc(), pos, vel, T, friction, dt, seed, n_steps));
}
int ocm_batch_admit_resume(ocm_batch* batch, const ocm_system* s, const double* pos, const double* vel,
                           double T, double friction, double dt, int32_t seed, int64_t n_steps,
                           int64_t steps_done, int64_t* slot_out) {
    BATCH_CALL(need(s, "system"); need(pos, "positions"); need(vel, "velocities"); need(slot_out, "slot_out");
               *slot_out = batch->b->admit(s->g.desc(), pos, vel, T, friction, dt, seed, n_steps, steps_done));
}
int ocm_batch_set_balanced(ocm_batch* batch, int on) { BATCH_CALL(batch->b->set_balanced(on != 0)); }
int ocm_batch_set_split(ocm_batch* batch, int32_t beads) { BATCH_CALL(batch->b->set_split(beads)); }
int ocm_batch_slot_status(ocm_batch* batch, int64_t slot, int32_t* status) {
    BATCH_CALL(need(status, "status"); *status = batch->b->slot_status(slot));
}
int ocm_batch_run(ocm_batch* batch, int32_t steps_per_launch, int sync) {
    BATCH_CALL(batch->b->run(steps_per_launch, sync != 0));
}
int ocm_batch_finished(ocm_batch* batch, int64_t* slots, int64_t cap, int64_t* n_out) {
    BATCH_CALL(need(n_out, "n_out"); batch->b->finished(slots, cap, n_out));
}
int ocm_batch_get_positions(ocm_batch* batch, int64_t slot, double* xyz) {
    BATCH_CALL(need(xyz, "xyz"); batch->b->get_positions(slot, xyz));
}
int ocm_batch_get_velocities(ocm_batch* batch, int64_t slot, double* v) {
    BATCH_CALL(need(v, "v"); batch->b->get_velocities(slot, v));
}
int ocm_batch_set_positions_many(ocm_batch* batch, int64_t n, const int64_t* slots,
                                 const double* xyz, const double* v) {
    BATCH_CALL(if (n) { need(slots, "slots"); need(xyz, "xyz"); }
               batch->b->set_positions_many(n, slots, xyz, v));
}
int ocm_batch_get_positions_many(ocm_batch* batch, int64_t n, const int64_t* slots, double* xyz) {
    BATCH_CALL(if (n) { need(slots, "slots"); need(xyz, "xyz"); }
               batch->b->get_positions_many(n, slots, xyz));
}
int ocm_batch_get_positions_many_noalloc(ocm_batch* batch, int64_t n, const int64_t* slots,
                                         double* xyz) {
    BATCH_CALL(if (n) { need(slots, "slots"); need(xyz, "xyz"); }
               batch->b->get_positions_many_noalloc(n, slots, xyz));
}
int ocm_batch_steps_done(ocm_batch* batch, int64_t slot, int64_t* steps) {
    BATCH_CALL(need(steps, "steps"); *steps = batch->b->steps_done(slot));
}
int ocm_batch_get_state(ocm_batch* batch, int64_t slot, uint32_t groups, double* forces,
                        double* energies) {
    BATCH_CALL(batch->b->get_state(slot, groups, forces, energies));
}
int ocm_batch_retire(ocm_batch* batch, int64_t slot) { BATCH_CALL(batch->b->retire(slot)); }
int ocm_batch_active(ocm_batch* batch, int64_t* n_active, int64_t* beads) {
    BATCH_CALL(need(n_active, "n_active"); need(beads, "beads");
               batch->b->active(n_active, beads));
}
int ocm_batch_last_run_ms(ocm_batch* batch, double* ms) {
    BATCH_CALL(need(ms, "ms"); *ms = batch->b->last_run_ms());
}
int ocm_batch_set_threads(ocm_batch* batch, int32_t threads) {
    BATCH_CALL(batch->b->set_threads(threads));
}
int ocm_batch_set_list_smem(ocm_batch* batch, int32_t kib) {
    BATCH_CALL(batch->b->set_list_smem(kib));
}
int ocm_batch_get_threads(ocm_batch* batch, int32_t* threads) {
    BATCH_CALL(need(threads, "threads"); *threads = batch->b->threads());
}
int ocm_batch_slot_stats(ocm_batch* batch, int64_t slot, int32_t* builds, int32_t* capacity) {
    BATCH_CALL(need(builds, "builds"); need(capacity, "capacity");
               batch->b->slot_stats(slot, builds, capacity));
}

}  // extern "C"
