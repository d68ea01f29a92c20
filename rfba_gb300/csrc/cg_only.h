// Gradient-only conjugate gradient in five dimensions, the optimiser 3B runs
// on each spot with the spot-gradient evaluation (RFBA Main/
// conjugate_gradient_only.h, driven as multispot5.cc:1624-1636 drives it).
//
// It never evaluates the function, only its gradient: the line search along
// the conjugate direction brackets the zero of the directional derivative,
// starting with the largest step the per-axis motion limits allow (halved
// while the gradient there is NaN), and narrows the bracket by secant steps
// once both ends have moved, bisection otherwise (conjugate_gradient_only.h:
// 106-230). Directions follow Polak-Ribiere (:250-270); the run stops after
// max_iterations line searches or when the largest gradient component falls
// under sqrt(machine epsilon) (:236-240). The arithmetic is kept in the
// reference's order (dot products summed from zero in index order, std::min /
// std::max comparison semantics, the step applied as x + s * direction), so
// with a bit-identical gradient the trajectory is bit-identical too; the
// translation unit that includes this is built without floating-point
// contraction. One deliberate difference: a line search whose allowed step is
// not finite (direction all zero or NaN) returns without moving instead of
// halving an infinite step forever.
//
// Licence and attribution. The step order above is that of B-cubed's
// conjugate_gradient_only.h, Copyright (C) 2009, 2010, 2011 Edward Rosten and
// Susan Cox, distributed under the GNU Lesser General Public License, version 3
// or (at your option) any later version. Because this header restates that
// algorithm step for step, it is offered under the same terms
// (LGPL-3.0-or-later); the rest of the library is unaffected.
#pragma once

#include <cmath>
#include <limits>

namespace rfba {

struct CgOnly5 {
    static constexpr int kMaxBracketSteps = 4096;
    double x[5], g[5], new_g[5], h[5], mh[5], dmax[5];
    double tolerance, ls_tolerance, ls_epsilon;
    int max_iterations, iterations, evaluations;

    static double dot(const double* a, const double* b) {
        double r = 0;
        for (int i = 0; i < 5; ++i) r += a[i] * b[i];
        return r;
    }
    static bool any_nan(const double* v) {
        for (int i = 0; i < 5; ++i)
            if (std::isnan(v[i])) return true;
        return false;
    }
    static double norm_inf(const double* v) {  // std::max(n, |v_i|) from |v_0|
        double n = std::fabs(v[0]);
        for (int i = 1; i < 5; ++i) {
            const double a = std::fabs(v[i]);
            n = (n < a) ? a : n;
        }
        return n;
    }

    // Gradient at x + s * mh into out; a non-zero return aborts the run.
    template <class Grad>
    int eval_along(Grad& grad, double s, double* out) {
        double p[5];
        for (int i = 0; i < 5; ++i) p[i] = x[i] + s * mh[i];
        ++evaluations;
        return grad(p, out);
    }

    template <class Grad>
    int start(const double s0[5], const double limit[5], Grad& grad) {
        const double eps = std::numeric_limits<double>::epsilon();
        for (int i = 0; i < 5; ++i) {
            x[i] = s0[i];
            dmax[i] = limit[i];
        }
        evaluations = 1;
        if (int e = grad(x, g)) return e;
        for (int i = 0; i < 5; ++i) {
            h[i] = g[i];
            mh[i] = -h[i];
        }
        tolerance = std::sqrt(eps);
        ls_tolerance = std::sqrt(eps);
        ls_epsilon = 1e-20;
        max_iterations = 5 * 100;
        iterations = 0;
        return 0;
    }

    // Restart from s0 with gvec taken as the gradient there, without an
    // evaluation (conjugate_gradient_only.h:65-86, init(start, deriv)).
    void restart(const double s0[5], const double gvec[5]) {
        const double eps = std::numeric_limits<double>::epsilon();
        for (int i = 0; i < 5; ++i) {
            x[i] = s0[i];
            g[i] = gvec[i];
            h[i] = g[i];
            mh[i] = -h[i];
        }
        tolerance = std::sqrt(eps);
        ls_tolerance = std::sqrt(eps);
        ls_epsilon = 1e-20;
        max_iterations = 5 * 100;
        iterations = 0;
    }

    template <class Grad>
    int line_search(Grad& grad) {
        ++iterations;
        for (int i = 0; i < 5; ++i) new_g[i] = g[i];
        double slope_lo = dot(g, mh);
        if (slope_lo > 0) return 0;  // not a descent direction: stay
        double step_cap = HUGE_VAL;
        for (int i = 0; i < 5; ++i) {
            const double v = std::fabs(dmax[i] / h[i]);
            step_cap = (v < step_cap) ? v : step_cap;
        }
        // With every direction component 0 or NaN the allowed step is not
        // finite; halving it never reaches the exit below and the reference's
        // search would not return. Stop this line search without moving.
        if (!(step_cap < HUGE_VAL)) return 0;
        const double first_step = step_cap;
        for (;;) {
            if (int e = eval_along(grad, step_cap, new_g)) return e;
            if (!any_nan(new_g)) break;
            step_cap /= 2;
            if (step_cap < first_step * ls_tolerance) return 0;
        }
        double slope_hi = dot(new_g, mh);
        if (slope_hi < 0) {  // still descending at the largest step: take it
            for (int i = 0; i < 5; ++i) x[i] += step_cap * mh[i];
            return 0;
        }
        double lo = 0, hi = step_cap, step = step_cap;
        int moved[2] = {0, 0};
        // the bracket shrinks every step (bisection at least every other one),
        // so the cap is never reached by a finite gradient; it only bounds the
        // host loop
        for (int n = 0; n < kMaxBracketSteps &&
                        std::fabs(lo - hi) > std::fabs(lo + hi) * ls_tolerance + ls_epsilon;
             ++n) {
            if (moved[0] != moved[1] && moved[0] != 0) {
                step = lo + slope_lo * (hi - lo) / (slope_lo - slope_hi);  // secant on the directional derivative
                if (int e = eval_along(grad, step, new_g)) return e;
                const double slope = dot(new_g, mh);
                moved[0] = moved[1];
                if (slope == 0) break;
                if (slope < 0) {
                    lo = step;
                    slope_lo = slope;
                    moved[1] = 1;
                } else {
                    hi = step;
                    slope_hi = slope;
                    moved[1] = 2;
                }
            } else {
                step = (lo + hi) / 2;
                if (int e = eval_along(grad, step, new_g)) return e;
                const double slope = dot(new_g, mh);
                if (slope < 0) {
                    lo = step;
                    slope_lo = slope;
                    moved[0] = 1;
                } else {
                    hi = step;
                    slope_hi = slope;
                    moved[0] = 2;
                }
            }
        }
        for (int i = 0; i < 5; ++i) x[i] += mh[i] * step;
        return 0;
    }

    bool finished() const { return iterations > max_iterations || norm_inf(new_g) < tolerance; }

    void update_polak_ribiere() {
        double old_g[5], old_h[5];
        for (int i = 0; i < 5; ++i) {
            old_g[i] = g[i];
            old_h[i] = h[i];
            g[i] = new_g[i];
        }
        const double gamma = (dot(g, g) - dot(old_g, g)) / dot(old_g, old_g);
        for (int i = 0; i < 5; ++i) {
            h[i] = g[i] + gamma * old_h[i];
            mh[i] = -h[i];
        }
    }

    // One iteration; *more is false once the run has finished.
    template <class Grad>
    int iterate(Grad& grad, bool* more) {
        if (int e = line_search(grad)) return e;
        *more = !finished();
        if (*more) update_polak_ribiere();
        return 0;
    }

    template <class Grad>
    int run(Grad& grad) {
        bool more = true;
        while (more)
            if (int e = iterate(grad, &more)) return e;
        return 0;
    }
};

}  // namespace rfba
