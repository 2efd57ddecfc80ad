// host_system.cpp - Topology, interaction groups, generators, SystemGenerator
// and the compile step.  Built with -ffp-contract=off so the generators'
// scans (FLA/FLD minimum energies) round exactly as written.
#include "host_system.hpp"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <sstream>
#include <tuple>

namespace ocm {

static std::string sz(std::size_t v) { return std::to_string(v); }

// ---------------------------------------------------------------------------
// Topology
// ---------------------------------------------------------------------------
int Topology::type_id(const std::string& type) {
    for (std::size_t i = 0; i < types_.size(); ++i)
        if (types_[i] == type) return (int)i;
    types_.push_back(type);
    return (int)types_.size() - 1;
}
int Topology::find_type(const std::string& type) const {
    for (std::size_t i = 0; i < types_.size(); ++i)
        if (types_[i] == type) return (int)i;
    return -1;
}

void Topology::add_edges(const std::vector<std::pair<std::size_t, std::size_t>>& edges,
                         const std::string& type) {
    const int t = type_id(type);
    for (const auto& e : edges) {
        if (e.first >= nodes_.size() || e.second >= nodes_.size())
            throw Error(1, "[error] Topology::add_edges: index out of range");
        nodes_[e.first].emplace_back(e.second, t);
        nodes_[e.second].emplace_back(e.first, t);
    }
    molecule_updated_ = false;
}

void Topology::make_molecule(const std::string& type) {
    // Depth-first flood fill over edges of `type`, seeded at the lowest
    // unvisited index (Topology.cpp:7-48).
    const int t = find_type(type);
    molecules_.clear();
    std::vector<char> seen(nodes_.size(), 0);
    std::size_t next = 0;
    std::vector<std::size_t> stack;
    while (true) {
        while (next < nodes_.size() && seen[next]) ++next;
        if (next == nodes_.size()) break;
        stack.push_back(next);
        molecules_.emplace_back();
        auto& mol = molecules_.back();
        while (!stack.empty()) {
            const std::size_t s = stack.back();
            stack.pop_back();
            mol.push_back(s);
            seen[s] = 1;
            for (const auto& e : nodes_[s])
                if (e.second == t && !seen[e.first]) stack.push_back(e.first);
        }
    }
    molecule_updated_ = true;
}

std::vector<std::pair<std::size_t, std::size_t>> Topology::ignore_list_within_molecule() const {
    if (!molecule_updated_)
        throw Error(5, "[error] ignore_list_within_molecule called before make_molecule");
    std::vector<std::pair<std::size_t, std::size_t>> out;
    for (const auto& mol : molecules_)
        for (std::size_t a = 0; a + 1 < mol.size(); ++a)
            for (std::size_t b = a + 1; b < mol.size(); ++b) out.emplace_back(mol[a], mol[b]);
    return out;
}

void Topology::collect_within(std::size_t node, std::size_t dist, int type,
                              std::vector<std::size_t>& out) const {
    // Recursive walk that records a node before descending and never
    // revisits a node already recorded (Topology.cpp:114-135).
    out.push_back(node);
    if (dist == 0) return;
    for (const auto& e : nodes_[node]) {
        if (e.second != type) continue;
        if (std::find(out.begin(), out.end(), e.first) == out.end())
            collect_within(e.first, dist - 1, type, out);
    }
}

std::vector<std::pair<std::size_t, std::size_t>> Topology::ignore_list_within_edge(
    std::size_t dist, const std::string& type) const {
    std::vector<std::pair<std::size_t, std::size_t>> out;
    const int t = find_type(type);
    if (t < 0) return out;
    std::vector<std::size_t> within;
    for (std::size_t i = 0; i < nodes_.size(); ++i) {
        within.clear();
        collect_within(i, dist, t, within);
        for (std::size_t j : within)
            if (j != i) out.emplace_back(std::min(i, j), std::max(i, j));
    }
    std::sort(out.begin(), out.end());
    out.erase(std::unique(out.begin(), out.end()), out.end());
    return out;
}

// ---------------------------------------------------------------------------
// Interaction groups
// ---------------------------------------------------------------------------
GroupPairs extract_interaction_group(const std::vector<bool>& has,
                                     const std::vector<std::pair<int, int>>& ignore_pairs,
                                     const std::vector<int>& group_vec) {
    GroupPairs out;
    if (ignore_pairs.empty()) {
        if (std::any_of(has.begin(), has.end(), [](bool b) { return !b; })) {
            std::set<int> part;
            for (std::size_t i = 0; i < has.size(); ++i)
                if (has[i]) part.insert((int)i);
            out.emplace_back(part, part);
        }
        return out;
    }
    std::set<int> related;
    for (const auto& p : ignore_pairs) {
        related.insert(p.first);
        related.insert(p.second);
    }
    std::map<int, std::set<int>> members;
    for (int g : related) members[g];
    std::set<int> others;
    for (std::size_t i = 0; i < has.size(); ++i) {
        if (!has[i]) continue;
        const int g = group_vec.empty() ? -1 : group_vec[i];
        if (g >= 0 && related.count(g))
            members[g].insert((int)i);
        else
            others.insert((int)i);
    }
    auto ignored = [&](int a, int b) {
        for (const auto& p : ignore_pairs)
            if ((p.first == a && p.second == b) || (p.first == b && p.second == a)) return true;
        return false;
    };
    out.emplace_back(others, others);
    std::vector<std::pair<int, std::set<int>>> vec(members.begin(), members.end());
    for (std::size_t i = 0; i < vec.size(); ++i) {
        out.emplace_back(vec[i].second, others);
        for (std::size_t j = i; j < vec.size(); ++j)
            if (!ignored(vec[i].first, vec[j].first)) out.emplace_back(vec[i].second, vec[j].second);
    }
    return out;
}

// ---------------------------------------------------------------------------
// Generators
// ---------------------------------------------------------------------------
HarmonicBondForceFieldGenerator::HarmonicBondForceFieldGenerator(
    std::vector<std::pair<int64_t, int64_t>> idx, std::vector<double> v0s, std::vector<double> ks,
    bool use_periodic)
    : idx_(std::move(idx)), v0s_(std::move(v0s)), ks_(std::move(ks)), periodic_(use_periodic) {
    if (!(idx_.size() == v0s_.size() && v0s_.size() == ks_.size()))
        throw Error(1, "[error] HarmonicBondForceFieldGenerator: parameter number of indices_vec (" +
                           sz(idx_.size()) + "), v0 (" + sz(v0s_.size()) + ") and k (" +
                           sz(ks_.size()) + ") is not matched.");
}
GeneratedForce HarmonicBondForceFieldGenerator::generate() const {
    GeneratedForce f;
    f.kind = ForceKind::HarmonicBond;
    f.name = name();
    f.periodic = periodic_;
    for (std::size_t i = 0; i < idx_.size(); ++i) {
        f.idx.push_back({idx_[i].first, idx_[i].second, -1, -1});
        f.par.push_back({v0s_[i], ks_[i]});
    }
    return f;
}

GoContactForceFieldGenerator::GoContactForceFieldGenerator(
    std::vector<std::pair<int64_t, int64_t>> idx, std::vector<double> ks, std::vector<double> r0s,
    bool use_periodic)
    : idx_(std::move(idx)), ks_(std::move(ks)), r0s_(std::move(r0s)), periodic_(use_periodic) {
    if (!(idx_.size() == ks_.size() && ks_.size() == r0s_.size()))
        throw Error(1, "[error] GoContactForceFieldGenerator : parameter number of indices_vec (" +
                           sz(idx_.size()) + "), k (" + sz(ks_.size()) + ") and r0 (" +
                           sz(r0s_.size()) + ") is not matched.");
}
GeneratedForce GoContactForceFieldGenerator::generate() const {
    GeneratedForce f;
    f.kind = ForceKind::GoContact;
    f.name = name();
    f.periodic = periodic_;
    for (std::size_t i = 0; i < idx_.size(); ++i) {
        f.idx.push_back({idx_[i].first, idx_[i].second, -1, -1});
        f.par.push_back({ks_[i], r0s_[i]});
    }
    return f;
}

GaussianBondForceFieldGenerator::GaussianBondForceFieldGenerator(
    std::vector<std::pair<int64_t, int64_t>> idx, std::vector<double> ks, std::vector<double> v0s,
    std::vector<double> sigmas, bool use_periodic)
    : idx_(std::move(idx)), ks_(std::move(ks)), v0s_(std::move(v0s)), sigmas_(std::move(sigmas)),
      periodic_(use_periodic) {
    if (!(idx_.size() == v0s_.size() && v0s_.size() == ks_.size() && ks_.size() == sigmas_.size()))
        throw Error(1, "[error] GaussianBondForceFieldGenerator: parameter number of indices_vec (" +
                           sz(idx_.size()) + "), k (" + sz(ks_.size()) + "), v0 (" + sz(v0s_.size()) +
                           ") and sigmas (" + sz(sigmas_.size()) +
                           ") is not matched.The number of these parameters must be same.");
}
GeneratedForce GaussianBondForceFieldGenerator::generate() const {
    GeneratedForce f;
    f.kind = ForceKind::GaussianBond;
    f.name = name();
    f.periodic = periodic_;
    for (std::size_t i = 0; i < idx_.size(); ++i) {
        f.idx.push_back({idx_[i].first, idx_[i].second, -1, -1});
        f.par.push_back({ks_[i], v0s_[i], sigmas_[i]});
    }
    return f;
}

GaussianDihedralForceFieldGenerator::GaussianDihedralForceFieldGenerator(
    std::vector<std::array<int64_t, 4>> idx, std::vector<double> ks, std::vector<double> theta0s,
    std::vector<double> sigmas, bool use_periodic)
    : idx_(std::move(idx)), ks_(std::move(ks)), theta0s_(std::move(theta0s)),
      sigmas_(std::move(sigmas)), periodic_(use_periodic) {
    if (!(idx_.size() == ks_.size() && idx_.size() == theta0s_.size() && idx_.size() == sigmas_.size()))
        throw Error(1, "[error] GaussianDihedralForceFieldGenerator : parameter number of indices_vec (" +
                           sz(idx_.size()) + "), k (" + sz(ks_.size()) + "), theta0 (" +
                           sz(theta0s_.size()) + ") and simga (" + sz(sigmas_.size()) +
                           " is not matched.The number of these parameters must be same.");
}
GeneratedForce GaussianDihedralForceFieldGenerator::generate() const {
    GeneratedForce f;
    f.kind = ForceKind::GaussianDihedral;
    f.name = name();
    f.periodic = periodic_;
    for (std::size_t i = 0; i < idx_.size(); ++i) {
        f.idx.push_back(idx_[i]);
        f.par.push_back({ks_[i], theta0s_[i], sigmas_[i]});
    }
    return f;
}

FlexibleLocalAngleForceFieldGenerator::FlexibleLocalAngleForceFieldGenerator(
    std::vector<std::array<int64_t, 3>> idx, std::vector<double> ks,
    const std::array<double, 10>& spline_table, const std::string& aa_name, bool use_periodic,
    double min_theta, double max_theta)
    : idx_(std::move(idx)), ks_(std::move(ks)), aa_(aa_name), min_theta_(min_theta),
      max_theta_(max_theta), dtheta_((max_theta - min_theta) / 9.0), rdtheta_(1.0 / dtheta_),
      y_(spline_table),
      thetas_{{1.30900, 1.48353, 1.65806, 1.83260, 2.00713, 2.18166, 2.35619, 2.53073, 2.70526,
               2.87979}},
      periodic_(use_periodic) {
    const auto* d2 = fla_second_derivative_table(aa_name);
    if (!d2) throw Error(1, "[error] FlexibleLocalAngleForceFieldGenerator: unknown amino acid " + aa_name);
    d2y_ = *d2;
    if (idx_.size() != ks_.size())
        throw Error(1, "[error] FlexibleLocalAngleForceFieldGenerator : parameter number ofindices_vec (" +
                           sz(idx_.size()) + ") and k (" + sz(ks_.size()) + ") is not matched.");
}

double FlexibleLocalAngleForceFieldGenerator::spline_interpolate(double th) const {
    // Same interval search and cubic as the reference's helper
    // (FlexibleLocalAngleForceFieldGenerator.cpp:47-68).
    constexpr double one_over_six = double(1.0) / double(6.0);
    std::size_t n = std::min<std::size_t>(8, (std::size_t)std::floor((th - min_theta_) * rdtheta_));
    if (thetas_[n + 1] < th) {
        n++;
    } else if (th < thetas_[n]) {
        n--;
    }
    const double a = (thetas_[n + 1] - th) * rdtheta_;
    const double b = (th - thetas_[n]) * rdtheta_;
    const double e1 = a * y_[n] + b * y_[n + 1];
    const double e2 = ((a * a * a - a) * d2y_[n] + (b * b * b - b) * d2y_[n + 1]) * dtheta_ *
                      dtheta_ * one_over_six;
    return e1 + e2;
}

GeneratedForce FlexibleLocalAngleForceFieldGenerator::generate() const {
    GeneratedForce f;
    f.kind = ForceKind::FlexibleLocalAngle;
    f.name = name();
    f.periodic = periodic_;
    double min_energy = y_[0];
    double th = min_theta_;
    while (th < max_theta_) {
        min_energy = std::min(min_energy, spline_interpolate(th));
        th += 1e-4;
    }
    f.spline_y = y_;
    f.theta_min = min_theta_;
    f.theta_max = max_theta_;
    f.min_energy = min_energy;
    for (std::size_t i = 0; i < idx_.size(); ++i) {
        f.idx.push_back({idx_[i][0], idx_[i][1], idx_[i][2], -1});
        f.par.push_back({ks_[i], 0.0});
    }
    return f;
}

FlexibleLocalDihedralForceFieldGenerator::FlexibleLocalDihedralForceFieldGenerator(
    std::vector<std::array<int64_t, 4>> idx, std::vector<double> ks,
    const std::array<double, 7>& fourier_table, const std::string& aa_pair_name, bool use_periodic)
    : idx_(std::move(idx)), ks_(std::move(ks)), f_(fourier_table), pair_(aa_pair_name),
      periodic_(use_periodic) {
    if (idx_.size() != ks_.size())
        throw Error(1, "[error] FlexibleLocalDihedralForceFieldGenerator : parameter number of indices_vec (" +
                           sz(idx_.size()) + ") and k (" + sz(ks_.size()) + ") is not matched.");
}

GeneratedForce FlexibleLocalDihedralForceFieldGenerator::generate() const {
    GeneratedForce f;
    f.kind = ForceKind::FlexibleLocalDihedral;
    f.name = name();
    f.periodic = periodic_;
    // Minimum of the Fourier series on a 1e-4 grid over [-pi, pi)
    // (FlexibleLocalDihedralForceFieldGenerator.cpp:7-26).
    double phi = -constant::pi;
    double min_energy = std::numeric_limits<double>::max();
    while (phi < constant::pi) {
        const double sin1 = std::sin(phi);
        const double cos1 = std::cos(phi);
        const double sin_sq = sin1 * sin1;
        const double cos_sq = cos1 * cos1;
        const double sin2 = 2 * sin1 * cos1;
        const double cos2 = cos_sq - sin_sq;
        const double sin3 = sin1 * (3 - 4 * sin_sq);
        const double cos3 = cos1 * (4 * cos_sq - 3);
        min_energy = std::min(min_energy, f_[1] * cos1 + f_[2] * sin1 + f_[3] * cos2 +
                                              f_[4] * sin2 + f_[5] * cos3 + f_[6] * sin3 + f_[0]);
        phi += 1e-4;
    }
    f.fourier = f_;
    f.min_energy = min_energy;
    for (std::size_t i = 0; i < idx_.size(); ++i) {
        f.idx.push_back({idx_[i][0], idx_[i][1], idx_[i][2], idx_[i][3]});
        f.par.push_back({ks_[i], 0.0});
    }
    return f;
}

static std::vector<bool> has_values(const std::vector<double>& v) {
    std::vector<bool> h(v.size());
    for (std::size_t i = 0; i < v.size(); ++i) h[i] = !std::isnan(v[i]);
    return h;
}

ExcludedVolumeForceFieldGenerator::ExcludedVolumeForceFieldGenerator(double eps, double cutoff,
                                                                     std::vector<double> radii,
                                                                     PairGeneratorCommon common)
    : eps_(eps), cutoff_(cutoff), radii_(std::move(radii)), c_(std::move(common)) {
    groups_ = extract_interaction_group(has_values(radii_), c_.ignore_group_pairs, c_.group_vec);
}
GeneratedForce ExcludedVolumeForceFieldGenerator::generate() const {
    GeneratedForce f;
    f.kind = ForceKind::ExcludedVolume;
    f.name = name();
    f.periodic = c_.use_periodic;
    double max_r = std::numeric_limits<double>::min();
    double second_r = std::numeric_limits<double>::min();
    for (double r : radii_) {
        if (std::isnan(r)) continue;
        if (max_r < r) {
            second_r = max_r;
            max_r = r;
        } else if (second_r < r) {
            second_r = r;
        }
    }
    f.cutoff = (max_r + second_r) * cutoff_;
    f.cutoff_correction = std::pow(1.0 / f.cutoff, 12);
    f.eps = eps_;
    f.pp0 = radii_;
    f.exclusions = c_.ignore_list;
    f.groups = groups_;
    return f;
}

double DebyeHuckelForceFieldGenerator::dielectric_water(double T, double C) {
    return (249.4 - 0.788 * T + 7.2e-4 * T * T) *
           (1. - 2.551e-1 * C + 5.151e-2 * C * C - 6.889e-3 * C * C * C);
}

DebyeHuckelForceFieldGenerator::DebyeHuckelForceFieldGenerator(double ionic_strength,
                                                               double temperature,
                                                               double cutoff_ratio,
                                                               std::vector<double> charges,
                                                               PairGeneratorCommon common)
    : ratio_(cutoff_ratio), q_(std::move(charges)), c_(std::move(common)) {
    // DebyeHuckelForceFieldGenerator.cpp:22-48
    const double epsk = dielectric_water(temperature, ionic_strength);
    const double eps0 = constant::eps0 / constant::elementary_charge / constant::elementary_charge;
    inv_4_pi_eps0_epsk_ = 1.0 / (4.0 * constant::pi * eps0 * epsk);
    if (!(ionic_strength > 0)) throw Error(1, "[error] ionic strength must be larger than zero");
    const double I = ionic_strength * 1.0e-24;
    debye_length_ = std::sqrt((eps0 * epsk * constant::kB * 1.0e-3 * temperature) / (2. * I));
    abs_cutoff_ = debye_length_ * ratio_;
    cutoff_correction_ = std::exp(-ratio_) / abs_cutoff_;
    groups_ = extract_interaction_group(has_values(q_), c_.ignore_group_pairs, c_.group_vec);
}
GeneratedForce DebyeHuckelForceFieldGenerator::generate() const {
    GeneratedForce f;
    f.kind = ForceKind::DebyeHuckel;
    f.name = name();
    f.periodic = c_.use_periodic;
    f.k_e = inv_4_pi_eps0_epsk_;
    f.debye_length = debye_length_;
    f.cutoff_correction = cutoff_correction_;
    f.cutoff = abs_cutoff_;
    f.pp0 = q_;
    f.exclusions = c_.ignore_list;
    f.groups = groups_;
    return f;
}

LennardJonesForceFieldGenerator::LennardJonesForceFieldGenerator(bool attractive, double ratio,
                                                                 std::vector<double> eps,
                                                                 std::vector<double> sigma,
                                                                 PairGeneratorCommon common)
    : attractive_(attractive), ratio_(ratio), eps_(std::move(eps)), sigma_(std::move(sigma)),
      c_(std::move(common)) {
    const std::string nm = attractive_ ? "LennardJonesAttractive" : "LennardJonesRepulsive";
    if (eps_.size() != sigma_.size())
        throw Error(1, nm + ": sigma.size(=" + sz(sigma_.size()) +
                           ") must be the same as epsilon.size(=" + sz(eps_.size()) + ")");
    for (std::size_t i = 0; i < eps_.size(); ++i)
        if (std::isnan(eps_[i]) != std::isnan(sigma_[i]))
            throw Error(1, nm + ": if particle i(=" + sz(i) +
                               ") has sigma, it should have epsilon too, and vice versa.");
    groups_ = extract_interaction_group(has_values(attractive_ ? eps_ : sigma_),
                                        c_.ignore_group_pairs, c_.group_vec);
}
GeneratedForce LennardJonesForceFieldGenerator::generate() const {
    GeneratedForce f;
    f.kind = attractive_ ? ForceKind::LennardJonesAttractive : ForceKind::LennardJonesRepulsive;
    f.name = name();
    f.periodic = c_.use_periodic;
    double max_s = std::numeric_limits<double>::min();
    double second_s = std::numeric_limits<double>::min();
    for (std::size_t i = 0; i < sigma_.size(); ++i) {
        if (std::isnan(sigma_[i])) continue;
        const double s = sigma_[i];
        if (max_s <= s) {
            second_s = max_s;
            max_s = s;
        } else if (second_s <= s) {
            second_s = s;
        }
    }
    f.cutoff = (max_s + second_s) * 0.5 * ratio_;
    if (attractive_) f.switch_distance = 0.9 * f.cutoff;
    f.pp0 = eps_;
    f.pp1 = sigma_;
    f.exclusions = c_.ignore_list;
    f.groups = groups_;
    return f;
}

// Largest and second-largest value of the defined entries (the reference's
// scan, which starts both from the smallest positive double).
static std::pair<double, double> two_largest(const std::vector<double>& v) {
    double m1 = std::numeric_limits<double>::min(), m2 = std::numeric_limits<double>::min();
    for (double s : v) {
        if (std::isnan(s)) continue;
        if (m1 <= s) {
            m2 = m1;
            m1 = s;
        } else if (m2 <= s) {
            m2 = s;
        }
    }
    return {m1, m2};
}

WeeksChandlerAndersenForceFieldGenerator::WeeksChandlerAndersenForceFieldGenerator(
    std::vector<double> sigmas, std::vector<double> eps, PairGeneratorCommon common)
    : sigma_(std::move(sigmas)), eps_(std::move(eps)), c_(std::move(common)) {
    if (sigma_.size() != eps_.size())
        throw Error(1, "WCA: sigma.size(=" + sz(sigma_.size()) + ") must be the same as epsilon.size(=" +
                           sz(eps_.size()) + ")");
    for (std::size_t i = 0; i < sigma_.size(); ++i) {
        if (std::isnan(sigma_[i]) != std::isnan(eps_[i]))
            throw Error(1, "WCA: if particle i(=" + sz(i) +
                               ") has sigma, it should have epsilon too, and vice versa.");
        if (eps_[i] < 0) throw Error(1, "WCA: epsilon of particle " + sz(i) + " is negative");
    }
    groups_ = extract_interaction_group(has_values(sigma_), c_.ignore_group_pairs, c_.group_vec);
}
GeneratedForce WeeksChandlerAndersenForceFieldGenerator::generate() const {
    GeneratedForce f;
    f.kind = ForceKind::WeeksChandlerAndersen;
    f.name = name();
    f.periodic = c_.use_periodic;
    const auto m = two_largest(sigma_);
    f.cutoff = (m.first + m.second) * 0.5 * std::pow(2.0, 1.0 / 6.0);
    f.pp0 = eps_;
    f.pp1 = sigma_;
    f.exclusions = c_.ignore_list;
    f.groups = groups_;
    return f;
}

// Interaction groups of a uniform generator between `former` and `latter`
// (UniformLennardJonesAttractiveForceFieldGenerator.cpp:28-138): without
// group-based ignores the one group (former, latter).  Otherwise each side
// splits into the members of every group named in an ignored pair and the
// rest ("others"); the groups are (others, named), (others, others),
// (named, others) and (named a, named b) unless (a, b) is ignored.
static GroupPairs uniform_groups(const std::vector<int64_t>& former, const std::vector<int64_t>& latter,
                                 const std::vector<std::pair<int, int>>& ignore_pairs,
                                 const std::vector<int>& group_vec) {
    GroupPairs out;
    auto as_set = [](const std::vector<int64_t>& v) {
        std::set<int> r;
        for (int64_t i : v) r.insert((int)i);
        return r;
    };
    if (ignore_pairs.empty()) {
        out.emplace_back(as_set(former), as_set(latter));
        return out;
    }
    std::set<int> related;
    for (const auto& p : ignore_pairs) {
        related.insert(p.first);
        related.insert(p.second);
    }
    auto split = [&](const std::vector<int64_t>& side, std::map<int, std::set<int>>& named,
                     std::set<int>& others) {
        for (int g : related) named[g];
        for (int64_t i : side) {
            const int g = group_vec.empty() ? -1 : group_vec[i];
            if (g >= 0 && related.count(g)) named[g].insert((int)i);
            else others.insert((int)i);
        }
    };
    std::map<int, std::set<int>> fnamed, lnamed;
    std::set<int> fothers, lothers;
    split(former, fnamed, fothers);
    split(latter, lnamed, lothers);
    auto push = [&](const std::set<int>& a, const std::set<int>& b) {
        if (!a.empty() && !b.empty()) out.emplace_back(a, b);  // an empty side adds no pair
    };
    if (!fothers.empty()) {
        for (const auto& l : lnamed) push(fothers, l.second);
        push(fothers, lothers);
    }
    for (const auto& f : fnamed) {
        push(f.second, lothers);
        for (const auto& l : lnamed) {
            const bool ignored = std::find(ignore_pairs.begin(), ignore_pairs.end(),
                                           std::make_pair(f.first, l.first)) != ignore_pairs.end();
            if (!ignored) push(f.second, l.second);
        }
    }
    return out;
}

UniformPairForceFieldGenerator::UniformPairForceFieldGenerator(bool attractive, int64_t system_size,
                                                               double eps, double sigma, double ratio,
                                                               std::vector<int64_t> former,
                                                               std::vector<int64_t> latter,
                                                               PairGeneratorCommon common)
    : attractive_(attractive), n_(system_size), eps_(eps), sigma_(sigma), ratio_(ratio),
      c_(std::move(common)) {
    if (!(sigma_ > 0)) throw Error(1, "[error] " + name() + ": sigma must be positive");
    if (!(eps_ >= 0)) throw Error(1, "[error] " + name() + ": epsilon must be >= 0");
    if (attractive_ && !(ratio_ > 0)) throw Error(1, "[error] " + name() + ": cutoff ratio must be positive");
    for (const auto* side : {&former, &latter})
        for (int64_t i : *side)
            if (i < 0 || i >= n_)
                throw Error(1, "[error] " + name() + " : index " + std::to_string(i) +
                                   " exceeds the system's largest index " + std::to_string(n_ - 1) + ".");
    groups_ = uniform_groups(former, latter, c_.ignore_group_pairs, c_.group_vec);
}
GeneratedForce UniformPairForceFieldGenerator::generate() const {
    GeneratedForce f;
    f.kind = attractive_ ? ForceKind::LennardJonesAttractive : ForceKind::LennardJonesRepulsive;
    f.name = name();
    f.periodic = c_.use_periodic;
    f.cutoff = attractive_ ? sigma_ * ratio_ : sigma_ * std::pow(2.0, 1.0 / 6.0);
    if (attractive_) f.switch_distance = 0.9 * f.cutoff;
    f.pp0.assign(n_, eps_);
    f.pp1.assign(n_, sigma_);
    f.exclusions = c_.ignore_list;
    f.groups = groups_;
    if (f.groups.empty()) f.groups.emplace_back(std::set<int>(), std::set<int>());  // nobody interacts
    return f;
}

CappedGoContactForceFieldGenerator::CappedGoContactForceFieldGenerator(
    std::vector<std::pair<int64_t, int64_t>> idx, std::vector<double> ks, std::vector<double> r0s,
    double capping_ratio, bool use_periodic)
    : idx_(std::move(idx)), ks_(std::move(ks)), r0s_(std::move(r0s)), cap_(capping_ratio),
      periodic_(use_periodic) {
    if (!(idx_.size() == ks_.size() && ks_.size() == r0s_.size()))
        throw Error(1, "[error] CappedGoContactForceFieldGenerator : parameter number of indices_vec (" +
                           sz(idx_.size()) + "), k (" + sz(ks_.size()) + ") and r0 (" + sz(r0s_.size()) +
                           ") is not matched.The number of these parameters must be same.");
    if (!(cap_ > 0)) throw Error(1, "[error] CappedGoContactForceFieldGenerator : capping ratio must be positive");
}
GeneratedForce CappedGoContactForceFieldGenerator::generate() const {
    GeneratedForce f;
    f.kind = ForceKind::CappedGoContact;
    f.name = name();
    f.periodic = periodic_;
    for (std::size_t i = 0; i < idx_.size(); ++i) {
        f.idx.push_back({idx_[i].first, idx_[i].second, -1, -1});
        f.par.push_back({ks_[i], r0s_[i], cap_});
    }
    return f;
}

// ---------------------------------------------------------------------------
// SystemGenerator
// ---------------------------------------------------------------------------
void SystemGenerator::set_pbc(double x, double y, double z) {
    if (!(x > 0 && y > 0 && z > 0)) throw Error(1, "[error] periodic box lengths must be positive");
    desc_.periodic_box = true;
    desc_.box[0] = x;
    desc_.box[1] = y;
    desc_.box[2] = z;
}

int SystemGenerator::add_ff_generator(std::unique_ptr<ForceFieldGeneratorBase> gen) {
    // One group per generator name, FLA / FLD families collapsed
    // (SystemGenerator.cpp:4-32, 69-85).
    const int next = (int)group_of_name_.size();
    const std::string nm = gen->name();
    std::string key = nm;
    if (nm.find("FlexibleLocalAngle") != std::string::npos) key = "FlexibleLocalAngle";
    else if (nm.find("FlexibleLocalDihedral") != std::string::npos) key = "FlexibleLocalDihedral";
    group_of_name_.insert({key, next});
    const int group = group_of_name_.at(key);
    if (group >= 32) throw Error(1, "[error] more than 32 force groups");
    GeneratedForce f = gen->generate();
    const int64_t n = (int64_t)desc_.masses.size();
    for (const auto& ix : f.idx)
        for (int64_t v : ix)
            if (v >= n) throw Error(1, "[error] " + nm + " : index " + std::to_string(v) +
                                           " exceeds the system's largest index " +
                                           std::to_string(n - 1) + ".");
    for (const auto& p : f.exclusions)
        if (p.first < 0 || p.second < 0 || p.first >= n || p.second >= n)
            throw Error(1, "[error] " + nm + " : exclusion index out of range");
    if (!f.pp0.empty() && (int64_t)f.pp0.size() != n)
        throw Error(1, "[error] " + nm + " : per-particle parameter count != system size");
    f.group = group;
    if ((int)desc_.group_names.size() <= group) desc_.group_names.resize(group + 1);
    desc_.group_names[group] = key;
    desc_.forces.push_back(std::move(f));
    return group;
}

std::string SystemGenerator::describe_json() const {
    std::ostringstream o;
    o.precision(17);
    o << "{\"n_particles\": " << desc_.masses.size() << ", \"periodic_box\": "
      << (desc_.periodic_box ? "true" : "false") << ", \"box\": [" << desc_.box[0] << ", "
      << desc_.box[1] << ", " << desc_.box[2] << "], \"forces\": [";
    bool first = true;
    for (const auto& f : desc_.forces) {
        if (!first) o << ", ";
        first = false;
        int64_t participants = 0;
        for (double v : f.pp0) participants += !std::isnan(v);
        o << "{\"name\": \"" << f.name << "\", \"group\": " << f.group
          << ", \"periodic\": " << (f.periodic ? "true" : "false") << ", \"terms\": " << f.idx.size()
          << ", \"cutoff\": " << f.cutoff << ", \"switch_distance\": " << f.switch_distance
          << ", \"eps\": " << f.eps << ", \"cutoff_correction\": " << f.cutoff_correction
          << ", \"k_e\": " << f.k_e << ", \"debye_length\": " << f.debye_length
          << ", \"min_energy\": " << f.min_energy << ", \"participants\": " << participants
          << ", \"exclusions\": " << f.exclusions.size()
          << ", \"interaction_groups\": " << f.groups.size() << "}";
    }
    o << "]}";
    return o.str();
}

// ---------------------------------------------------------------------------
// Compile
// ---------------------------------------------------------------------------
std::array<double, 10> natural_spline_second_derivatives(const std::array<double, 10>& y,
                                                         double h) {
    // M0 = M9 = 0; M[k-1] + 4 M[k] + M[k+1] = 6 (y[k+1] - 2 y[k] + y[k-1]) / h^2.
    std::array<double, 10> M{};
    double c[10] = {0}, d[10] = {0};
    for (int k = 1; k <= 8; ++k) {
        const double rhs = 6.0 * (y[k + 1] - 2.0 * y[k] + y[k - 1]) / (h * h);
        const double denom = 4.0 - (k > 1 ? c[k - 1] : 0.0);
        c[k] = 1.0 / denom;
        d[k] = (rhs - (k > 1 ? d[k - 1] : 0.0)) / denom;
    }
    M[8] = d[8];
    for (int k = 7; k >= 1; --k) M[k] = d[k] - c[k] * M[k + 1];
    return M;
}

namespace {

struct LabelResult {
    std::vector<uint8_t> label;
    unsigned long long allow = 0;
};

LabelResult make_labels(const GroupPairs& groups, const std::vector<double>& values, int64_t n,
                        const std::string& nm) {
    LabelResult r;
    r.label.assign(n, 0);
    if (groups.empty()) {
        for (int64_t i = 0; i < n; ++i)
            if (!values.empty() && std::isnan(values[i]))
                throw Error(1, "[error] " + nm + ": particle " + std::to_string(i) +
                                   " has no parameter but no interaction group excludes it");
        r.allow = 1ull;
        return r;
    }
    const std::size_t G = groups.size();
    std::vector<std::vector<char>> in1(G, std::vector<char>(n, 0)), in2(G, std::vector<char>(n, 0));
    for (std::size_t g = 0; g < G; ++g) {
        for (int p : groups[g].first) in1[g][p] = 1;
        for (int p : groups[g].second) in2[g][p] = 1;
    }
    std::map<std::vector<char>, int> sig_label;
    std::vector<int64_t> rep;
    for (int64_t i = 0; i < n; ++i) {
        std::vector<char> sig(2 * G);
        bool any = false;
        for (std::size_t g = 0; g < G; ++g) {
            sig[2 * g] = in1[g][i];
            sig[2 * g + 1] = in2[g][i];
            any = any || in1[g][i] || in2[g][i];
        }
        if (!any) {
            r.label[i] = 15;
            continue;
        }
        auto it = sig_label.find(sig);
        if (it == sig_label.end()) {
            const int l = (int)sig_label.size();
            if (l >= 8)
                throw Error(6, "[error] " + nm + ": more than 8 distinct interaction-group memberships");
            it = sig_label.emplace(sig, l).first;
            rep.push_back(i);
        }
        r.label[i] = (uint8_t)it->second;
    }
    const int L = (int)rep.size();
    for (int a = 0; a < L; ++a)
        for (int b = 0; b < L; ++b) {
            int count = 0;
            for (std::size_t g = 0; g < G; ++g)
                count += (in1[g][rep[a]] && in2[g][rep[b]]) || (in2[g][rep[a]] && in1[g][rep[b]]);
            if (count > 1)
                throw Error(6, "[error] " + nm + ": a particle pair lies in more than one interaction group");
            if (count) r.allow |= 1ull << (a * 8 + b);
        }
    return r;
}

}  // namespace

CompiledSystem compile_system(const SystemDesc& d) {
    CompiledSystem c;
    const int64_t n = (int64_t)d.masses.size();
    c.n = n;
    c.inv_mass.resize(n);
    for (int64_t i = 0; i < n; ++i) {
        if (!(d.masses[i] >= 0)) throw Error(1, "[error] particle masses must be >= 0");
        c.inv_mass[i] = d.masses[i] > 0 ? (float)(1.0 / d.masses[i]) : 0.f;
    }
    c.p0.assign(4 * n, 0.f);
    c.p1.assign(4 * n, 0.f);
    c.labels.assign(n, 0u);
    for (int s = 0; s < kNumSlots; ++s) c.slot_group[s] = -1;
    std::memset(&c.pc, 0, sizeof(c.pc));
    c.box[0] = d.box[0];
    c.box[1] = d.box[1];
    c.box[2] = d.box[2];

    int pair_periodic = -1;
    // exclusion triples (i, j, bit)
    std::vector<std::tuple<int32_t, int32_t, uint8_t>> ex;
    for (const auto& f : d.forces) {
        int term = -1, slot = -1;
        switch (f.kind) {
            case ForceKind::ExcludedVolume: term = 0; slot = kSlotEXV; break;
            case ForceKind::DebyeHuckel: term = 1; slot = kSlotDH; break;
            case ForceKind::LennardJonesRepulsive: term = 2; slot = kSlotLJR; break;
            case ForceKind::WeeksChandlerAndersen: term = 2; slot = kSlotLJR; break;
            case ForceKind::CappedGoContact: slot = kSlotCGO; break;
            case ForceKind::LennardJonesAttractive: term = 3; slot = kSlotLJA; break;
            case ForceKind::HarmonicBond: slot = kSlotHB; break;
            case ForceKind::GoContact: slot = kSlotGO; break;
            case ForceKind::FlexibleLocalAngle: slot = kSlotFLA; break;
            case ForceKind::FlexibleLocalDihedral: slot = kSlotFLD; break;
            case ForceKind::GaussianBond: slot = kSlotGB; break;
            case ForceKind::GaussianDihedral: slot = kSlotGD; break;
        }
        if (term >= 0) {
            const int bit = 1 << term;
            if ((c.pc.terms & bit) && term == 2)
                throw Error(6, "[error] " + f.name + ": LennardJonesRepulsive, WeeksChandlerAndersen and "
                               "UniformWeeksChadlerAndersen share one pair slot; a system holds at most one of them");
            if (c.pc.terms & bit)
                throw Error(6, "[error] more than one " + f.name + " force in one system");
            if (f.kind == ForceKind::WeeksChandlerAndersen) c.pc.ljr_geometric = 1;
            c.pc.terms |= bit;
            if (pair_periodic >= 0 && pair_periodic != (int)f.periodic)
                throw Error(6, "[error] pair forces mix periodic and non-periodic cutoffs");
            pair_periodic = f.periodic;
            if (f.periodic && !d.periodic_box)
                throw Error(1, "[error] " + f.name + " uses periodic cutoffs but no box was set");
            if (!(f.cutoff > 0) || !std::isfinite(f.cutoff))
                throw Error(1, "[error] " + f.name + " cutoff must be positive");
            if (f.periodic)
                for (int a = 0; a < 3; ++a)
                    if (f.cutoff > 0.5 * d.box[a])
                        throw Error(1, "[error] " + f.name +
                                           " cutoff exceeds half the periodic box length");
            // A Debye-Hueckel group that only separates charged from uncharged
            // particles needs no labels: an uncharged particle carries q = 0
            // and contributes nothing.
            GroupPairs groups = f.groups;
            if (f.kind == ForceKind::DebyeHuckel && groups.size() == 1 &&
                groups[0].first == groups[0].second) {
                std::set<int> part;
                for (int64_t i = 0; i < n; ++i)
                    if (!std::isnan(f.pp0[i])) part.insert((int)i);
                if (part == groups[0].first) groups.clear();
            }
            std::vector<double> flagv = f.pp0;
            if (f.kind == ForceKind::DebyeHuckel && groups.empty())
                for (auto& v : flagv)
                    if (std::isnan(v)) v = 0.0;
            LabelResult lr = make_labels(groups, flagv, n, f.name);
            for (int64_t i = 0; i < n; ++i) {
                c.labels[i] |= (uint32_t)lr.label[i] << (4 * term);
                const bool part = lr.label[i] != 15;
                double a = f.pp0.empty() ? 0.0 : f.pp0[i];
                if (f.kind == ForceKind::DebyeHuckel && std::isnan(a) && groups.empty()) a = 0.0;
                const double b = f.pp1.empty() ? 0.0 : f.pp1[i];
                if (part && (std::isnan(a) || std::isnan(b)))
                    throw Error(1, "[error] " + f.name + ": participating particle " +
                                       std::to_string(i) + " has NaN parameters");
                switch (f.kind) {
                    case ForceKind::ExcludedVolume: c.p0[4 * i + 0] = part ? (float)a : 0.f; break;
                    case ForceKind::DebyeHuckel: c.p0[4 * i + 1] = part ? (float)a : 0.f; break;
                    case ForceKind::LennardJonesRepulsive:
                        c.p0[4 * i + 2] = part ? (float)a : 0.f;
                        c.p0[4 * i + 3] = part ? (float)b : 0.f;
                        break;
                    case ForceKind::WeeksChandlerAndersen:  // sqrt(eps): the kernel multiplies
                        c.p0[4 * i + 2] = part ? (float)std::sqrt(a) : 0.f;
                        c.p0[4 * i + 3] = part ? (float)b : 0.f;
                        break;
                    case ForceKind::LennardJonesAttractive:
                        c.p1[4 * i + 0] = part ? (float)a : 0.f;
                        c.p1[4 * i + 1] = part ? (float)b : 0.f;
                        break;
                    default: break;
                }
            }
            c.pc.allow[term] = lr.allow;
            if (!groups.empty()) c.pc.uses_labels |= bit;
            const double rc = f.cutoff;
            const float rc2 = (float)(rc * rc);
            switch (f.kind) {
                case ForceKind::ExcludedVolume:
                    c.pc.exv_eps = (float)f.eps;
                    c.pc.exv_rc2 = rc2;
                    c.pc.exv_inv_rc2 = (float)(1.0 / (rc * rc));
                    break;
                case ForceKind::DebyeHuckel:
                    c.pc.dh_k = (float)f.k_e;
                    c.pc.dh_inv_lambda = (float)(1.0 / f.debye_length);
                    c.pc.dh_inv_lambda_log2e = (float)(1.4426950408889634 / f.debye_length);
                    c.pc.dh_rc2 = rc2;
                    c.pc.dh_corr = (float)f.cutoff_correction;
                    break;
                case ForceKind::LennardJonesRepulsive:
                case ForceKind::WeeksChandlerAndersen: c.pc.ljr_rc2 = rc2; break;
                case ForceKind::LennardJonesAttractive:
                    c.pc.lja_rc2 = rc2;
                    c.pc.lja_rs = (float)f.switch_distance;
                    c.pc.lja_inv_width = (float)(1.0 / (rc - f.switch_distance));
                    break;
                default: break;
            }
            c.max_cutoff = std::max(c.max_cutoff, rc);
            for (const auto& p : f.exclusions) {
                if (p.first == p.second) continue;
                ex.emplace_back((int32_t)p.first, (int32_t)p.second, (uint8_t)bit);
                ex.emplace_back((int32_t)p.second, (int32_t)p.first, (uint8_t)bit);
            }
        } else if (f.kind == ForceKind::HarmonicBond || f.kind == ForceKind::GoContact) {
            for (std::size_t t = 0; t < f.idx.size(); ++t) {
                BondTerm b;
                b.i = (int32_t)f.idx[t][0];
                b.j = (int32_t)f.idx[t][1];
                b.kind = f.kind == ForceKind::HarmonicBond ? kBondHarmonic : kBondGo;
                b.periodic = f.periodic ? 1 : 0;
                b.p0 = (float)f.par[t][0];
                b.p1 = (float)f.par[t][1];
                const double r0 = f.kind == ForceKind::HarmonicBond ? f.par[t][0] : f.par[t][1];
                const double r0sq = r0 * r0;
                b.r0sq_hi = (float)r0sq;
                b.r0sq_lo = (float)(r0sq - (double)b.r0sq_hi);
                if (b.i < 0 || b.j < 0) throw Error(1, "[error] negative particle index");
                c.bonds.push_back(b);
            }
        } else if (f.kind == ForceKind::CappedGoContact) {
            for (std::size_t t = 0; t < f.idx.size(); ++t) {
                BondTerm b{};
                b.i = (int32_t)f.idx[t][0];
                b.j = (int32_t)f.idx[t][1];
                b.kind = kBondCappedGo;
                b.periodic = f.periodic ? 1 : 0;
                b.p0 = (float)f.par[t][0];                // k
                b.p1 = (float)(1.0 / f.par[t][2]);        // 1 / capping ratio
                const double r0sq = f.par[t][1] * f.par[t][1];
                b.r0sq_hi = (float)r0sq;
                b.r0sq_lo = (float)(r0sq - (double)b.r0sq_hi);
                if (b.i < 0 || b.j < 0) throw Error(1, "[error] negative particle index");
                c.bonds.push_back(b);
            }
        } else if (f.kind == ForceKind::GaussianBond) {
            for (std::size_t t = 0; t < f.idx.size(); ++t) {
                BondTerm b{};
                b.i = (int32_t)f.idx[t][0];
                b.j = (int32_t)f.idx[t][1];
                b.kind = kBondGauss;
                b.periodic = f.periodic ? 1 : 0;
                b.p0 = (float)f.par[t][0];                                  // k
                b.p1 = (float)(1.0 / (2.0 * f.par[t][2] * f.par[t][2]));  // 1 / (2 sigma^2)
                const double v0sq = f.par[t][1] * f.par[t][1];
                b.r0sq_hi = (float)v0sq;
                b.r0sq_lo = (float)(v0sq - (double)b.r0sq_hi);
                if (b.i < 0 || b.j < 0) throw Error(1, "[error] negative particle index");
                c.bonds.push_back(b);
            }
        } else if (f.kind == ForceKind::GaussianDihedral) {
            for (std::size_t a = 0; a < f.idx.size(); ++a) {
                DihedralTerm dt{};
                dt.i = (int32_t)f.idx[a][0];
                dt.j = (int32_t)f.idx[a][1];
                dt.k = (int32_t)f.idx[a][2];
                dt.l = (int32_t)f.idx[a][3];
                if (dt.i < 0 || dt.j < 0 || dt.k < 0 || dt.l < 0)
                    throw Error(1, "[error] negative particle index");
                dt.kind = kDihGauss;
                dt.table = -1;
                dt.periodic = f.periodic ? 1 : 0;
                dt.kk = (float)f.par[a][0];
                dt.theta0 = (float)f.par[a][1];
                dt.inv2s2 = (float)(1.0 / (2.0 * f.par[a][2] * f.par[a][2]));
                c.dihedrals.push_back(dt);
            }
        } else if (f.kind == ForceKind::FlexibleLocalAngle) {
            FlaTable t{};
            const double h = (f.theta_max - f.theta_min) / 9.0;
            const auto M = natural_spline_second_derivatives(f.spline_y, h);
            t.theta_min = (float)f.theta_min;
            t.theta_max = (float)f.theta_max;
            t.inv_h = (float)(1.0 / h);
            t.emin = (float)f.min_energy;
            for (int k = 0; k < 10; ++k) {
                t.y[k] = (float)f.spline_y[k];
                t.m[k] = (float)(M[k] * h * h / 6.0);
            }
            const int tid = (int)c.fla.size();
            c.fla.push_back(t);
            for (std::size_t a = 0; a < f.idx.size(); ++a) {
                AngleTerm at;
                at.i = (int32_t)f.idx[a][0];
                at.j = (int32_t)f.idx[a][1];
                at.k = (int32_t)f.idx[a][2];
                if (at.i < 0 || at.j < 0 || at.k < 0) throw Error(1, "[error] negative particle index");
                at.table = tid;
                at.kk = (float)f.par[a][0];
                at.periodic = f.periodic ? 1 : 0;
                c.angles.push_back(at);
            }
        } else {
            FldTable t{};
            for (int k = 0; k < 7; ++k) t.c[k] = (float)f.fourier[k];
            t.emin = (float)f.min_energy;
            const int tid = (int)c.fld.size();
            c.fld.push_back(t);
            for (std::size_t a = 0; a < f.idx.size(); ++a) {
                DihedralTerm dt{};
                dt.i = (int32_t)f.idx[a][0];
                dt.j = (int32_t)f.idx[a][1];
                dt.k = (int32_t)f.idx[a][2];
                dt.l = (int32_t)f.idx[a][3];
                if (dt.i < 0 || dt.j < 0 || dt.k < 0 || dt.l < 0)
                    throw Error(1, "[error] negative particle index");
                dt.kind = kDihFLD;
                dt.table = tid;
                dt.periodic = f.periodic ? 1 : 0;
                dt.kk = (float)f.par[a][0];
                c.dihedrals.push_back(dt);
            }
        }
        if (c.slot_group[slot] >= 0 && c.slot_group[slot] != f.group)
            throw Error(6, "[error] forces of one kind placed in different groups");
        c.slot_group[slot] = f.group;
    }
    // Labels of absent terms: everybody participates (unused anyway).
    for (int t = 0; t < kNumPairTerms; ++t)
        if (!(c.pc.terms & (1 << t))) c.pc.allow[t] = 1ull;
    c.periodic = pair_periodic == 1;
    if (d.periodic_box) {
        c.box[0] = d.box[0];
        c.box[1] = d.box[1];
        c.box[2] = d.box[2];
    }
    for (const auto& b : c.bonds)
        if (b.periodic && !d.periodic_box) throw Error(1, "[error] periodic bond force without a box");
    c.pc.list_rc2 = (float)(c.max_cutoff * c.max_cutoff);
    if ((c.pc.terms & kTermLJR) && (c.pc.terms & kTermLJA)) {
        c.lj_same_sigma = true;
        for (int64_t i = 0; i < n && c.lj_same_sigma; ++i)
            c.lj_same_sigma = c.p0[4 * i + 3] == c.p1[4 * i + 1];
    }

    std::sort(ex.begin(), ex.end());
    c.ex_start.assign(n + 1, 0);
    for (std::size_t k = 0; k < ex.size();) {
        const int32_t i = std::get<0>(ex[k]), j = std::get<1>(ex[k]);
        uint8_t bits = 0;
        while (k < ex.size() && std::get<0>(ex[k]) == i && std::get<1>(ex[k]) == j)
            bits |= std::get<2>(ex[k++]);
        c.ex_j.push_back(j);
        c.ex_bits.push_back(bits);
        c.ex_start[i + 1]++;
    }
    for (int64_t i = 0; i < n; ++i) c.ex_start[i + 1] += c.ex_start[i];
    return c;
}

}  // namespace ocm
