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

    template <class Grad>
    int line_search(Grad& grad) {
        ++iterations;
        for (int i = 0; i < 5; ++i) new_g[i] = g[i];
        double f1 = dot(g, mh);
        if (f1 > 0) return 0;  // not a descent direction: stay
        double max_step = HUGE_VAL;
        for (int i = 0; i < 5; ++i) {
            const double v = std::fabs(dmax[i] / h[i]);
            max_step = (v < max_step) ? v : max_step;
        }
        // With every direction component 0 or NaN the allowed step is not
        // finite; halving it never reaches the exit below and the reference's
        // search would not return. Stop this line search without moving.
        if (!(max_step < HUGE_VAL)) return 0;
        const double full_max_step = max_step;
        for (;;) {
            if (int e = eval_along(grad, max_step, new_g)) return e;
            if (!any_nan(new_g)) break;
            max_step /= 2;
            if (max_step < full_max_step * ls_tolerance) return 0;
        }
        double f2 = dot(new_g, mh);
        if (f2 < 0) {  // still descending at the largest step: take it
            for (int i = 0; i < 5; ++i) x[i] += max_step * mh[i];
            return 0;
        }
        double s1 = 0, s2 = max_step, s_new = max_step;
        int updates[2] = {0, 0};
        // the bracket shrinks every step (bisection at least every other one),
        // so the cap is never reached by a finite gradient; it only bounds the
        // host loop
        for (int n = 0; n < kMaxBracketSteps &&
                        std::fabs(s1 - s2) > std::fabs(s1 + s2) * ls_tolerance + ls_epsilon;
             ++n) {
            if (updates[0] != updates[1] && updates[0] != 0) {
                s_new = s1 + f1 * (s2 - s1) / (f1 - f2);  // secant on the directional derivative
                if (int e = eval_along(grad, s_new, new_g)) return e;
                const double f_new = dot(new_g, mh);
                updates[0] = updates[1];
                if (f_new == 0) break;
                if (f_new < 0) {
                    s1 = s_new;
                    f1 = f_new;
                    updates[1] = 1;
                } else {
                    s2 = s_new;
                    f2 = f_new;
                    updates[1] = 2;
                }
            } else {
                s_new = (s1 + s2) / 2;
                if (int e = eval_along(grad, s_new, new_g)) return e;
                const double f_new = dot(new_g, mh);
                if (f_new < 0) {
                    s1 = s_new;
                    f1 = f_new;
                    updates[0] = 1;
                } else {
                    s2 = s_new;
                    f2 = f_new;
                    updates[0] = 2;
                }
            }
        }
        for (int i = 0; i < 5; ++i) x[i] += mh[i] * s_new;
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
