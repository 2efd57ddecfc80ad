// minimize.cpp - local energy minimisation of a plain context.
//
// The reference minimises once before its run when the input asks for it
// (Simulator.cpp:41-46, OpenMM::LocalEnergyMinimizer::minimize with the
// default tolerance of 10 kJ/mol/nm and no iteration limit).  This is a
// limited-memory BFGS (Nocedal & Wright, "Numerical Optimization", 2nd ed.,
// Algorithm 7.4, two-loop recursion, memory 10) on the FP64 master
// positions.  Energies and forces come from the context's device
// evaluation; the search stops once the root-mean-square of all force
// components is at most the tolerance.  A backtracking line search
// (sufficient decrease, c1 = 1e-4) whose first trial moves no bead further
// than 0.1 nm keeps the steps safe from overlapping configurations.  The
// search also ends when no step lowers the energy any more (the FP32 force
// noise floor), so a tolerance below that floor cannot loop forever; why
// it stopped (converged, iteration cap, stagnation, failed line search) and
// the final RMS force are kept for ocm_context_minimize_report.  A trial
// position whose evaluation blows up (a force of 1e9 kJ/mol/nm or more)
// counts as infinite energy, so the line search backs off from it.
#include <algorithm>
#include <cmath>
#include <deque>
#include <limits>
#include <vector>

#include "engine.hpp"

namespace ocm {

namespace {

double dot(const std::vector<double>& a, const std::vector<double>& b) {
    double s = 0;
    for (std::size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
    return s;
}

}  // namespace

int64_t PlainContext::minimize(double tolerance, int64_t max_iterations) {
    if (!(tolerance > 0)) throw Error(1, "[error] minimisation tolerance must be positive");
    if (max_iterations < 0) throw Error(1, "[error] maximum iteration count must be >= 0");
    check_positions_set();
    const std::size_t m3 = (std::size_t)(3 * n);
    std::vector<double> x(m3), g(m3), f(m3);
    get_positions(x.data());
    auto evaluate = [&](const std::vector<double>& pos, std::vector<double>& grad) {
        set_positions_internal(pos.data());
        double e = 0;
        try {
            get_state(0xffffffffu, f.data(), &e);
        } catch (const Error& err) {
            if (err.code != 7) throw;
            e = std::numeric_limits<double>::infinity();
        }
        for (std::size_t i = 0; i < m3; ++i) grad[i] = -f[i];
        return e;
    };
    auto rms = [&](const std::vector<double>& grad) { return std::sqrt(dot(grad, grad) / (double)m3); };

    double e = evaluate(x, g);
    if (!std::isfinite(e)) {
        set_positions_internal(x.data());
        throw Error(7, "[error] the starting positions give a non-finite energy or a force of 1e9 kJ/mol/nm "
                       "or more; minimisation cannot start");
    }
    min_reason = kMinIterationCap;
    std::deque<std::vector<double>> S, Y;
    std::deque<double> R;
    const std::size_t memory = 10;
    std::vector<double> p(m3), xn(m3), gn(m3), q(m3);
    int64_t it = 0;
    int failures = 0, stalled = 0;
    while (std::isfinite(e) && rms(g) > tolerance && (max_iterations == 0 || it < max_iterations)) {
        // two-loop recursion: p = -H g
        q = g;
        std::vector<double> alpha(S.size());
        for (std::size_t k = S.size(); k-- > 0;) {
            alpha[k] = R[k] * dot(S[k], q);
            for (std::size_t i = 0; i < m3; ++i) q[i] -= alpha[k] * Y[k][i];
        }
        const double gamma = S.empty() ? 1.0 : dot(S.back(), Y.back()) / dot(Y.back(), Y.back());
        for (std::size_t i = 0; i < m3; ++i) q[i] *= gamma;
        for (std::size_t k = 0; k < S.size(); ++k) {
            const double beta = R[k] * dot(Y[k], q);
            for (std::size_t i = 0; i < m3; ++i) q[i] += S[k][i] * (alpha[k] - beta);
        }
        for (std::size_t i = 0; i < m3; ++i) p[i] = -q[i];
        double slope = dot(g, p);
        if (!(slope < 0)) {  // not a descent direction: restart from steepest descent
            S.clear();
            Y.clear();
            R.clear();
            for (std::size_t i = 0; i < m3; ++i) p[i] = -g[i];
            slope = dot(g, p);
        }
        double pmax = 0;
        for (int64_t b = 0; b < n; ++b)
            pmax = std::max(pmax, std::sqrt(p[3 * b] * p[3 * b] + p[3 * b + 1] * p[3 * b + 1] +
                                             p[3 * b + 2] * p[3 * b + 2]));
        double step = pmax > 0.1 ? 0.1 / pmax : 1.0;
        double en = 0;
        bool accepted = false;
        for (int ls = 0; ls < 30; ++ls) {
            for (std::size_t i = 0; i < m3; ++i) xn[i] = x[i] + step * p[i];
            en = evaluate(xn, gn);
            if (std::isfinite(en) && en <= e + 1e-4 * step * slope) {
                accepted = true;
                break;
            }
            step *= 0.5;
        }
        ++it;
        if (!accepted) {
            // no decrease along this direction: forget the curvature pairs
            // and try steepest descent once more, then give up
            set_positions_internal(x.data());
            if (S.empty() || ++failures > 1) {
                min_reason = kMinLineSearch;
                break;
            }
            S.clear();
            Y.clear();
            R.clear();
            continue;
        }
        failures = 0;
        std::vector<double> s(m3), y(m3);
        for (std::size_t i = 0; i < m3; ++i) {
            s[i] = xn[i] - x[i];
            y[i] = gn[i] - g[i];
        }
        const double sy = dot(s, y);
        if (sy > 1e-12 * std::sqrt(dot(s, s) * dot(y, y))) {  // keep only positive curvature
            S.push_back(std::move(s));
            Y.push_back(std::move(y));
            R.push_back(1.0 / sy);
            if (S.size() > memory) {
                S.pop_front();
                Y.pop_front();
                R.pop_front();
            }
        }
        // FP32 forces put a floor under the reachable RMS force: stop once
        // 20 accepted steps in a row change the energy by less than 1e-12
        // relative, whatever the tolerance asked for
        stalled = std::fabs(en - e) <= 1e-12 * std::max(1.0, std::fabs(e)) ? stalled + 1 : 0;
        x.swap(xn);
        g.swap(gn);
        e = en;
        if (stalled >= 20) {
            min_reason = kMinStagnated;
            break;
        }
    }
    set_positions_internal(x.data());
    min_rms = rms(g);
    if (min_rms <= tolerance) min_reason = kMinConverged;
    return it;
}

}  // namespace ocm
