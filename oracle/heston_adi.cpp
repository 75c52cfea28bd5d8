// TEST INFRASTRUCTURE: the Heston ADI finite-difference price that judges the GPU
// least-squares Monte Carlo (American and European vanilla options under Heston).
//
// Restates kiyosi's FiniteDifferenceHestonVanillaEngine for flat rate and dividend
// curves (crates/kiyosi/src/engines/finite_difference/heston.rs):
//   * grid preparation: prepare_batch (heston.rs:650-996): scaled units, asset bounds
//     from integrated variance (analytic/heston.rs:436-455), spot_floor and the
//     log-spot SpatialGrid with sinh concentration at the strike (grid.rs:80-86,
//     222-336, 680-781), the sinh variance grid with the initial variance as a node
//     (heston.rs:405-440, 905-934), the uniform time grid (grid.rs:930-1022);
//   * operators: moment-matched log-spot stencils (grid.rs:104-200), upwinded
//     variance rows (heston.rs:1571-1586), nine-point mixed derivative
//     (heston.rs:1588-1596, 1900-1956), the discount split half per direction
//     (heston.rs:1725-1881);
//   * time stepping: modified Craig-Sneyd with theta = 1/3 in increment form
//     (heston.rs:1140-1190, 1958-2041, 2285-2347), Ikonen-Toivanen American splitting
//     (heston.rs:2043-2103), Dirichlet asset edges from the exercise-boundary rules
//     (deterministic.rs:333-363, 386-531), a Neumann top variance row;
//   * read-out: the valuation row's cubic spline in log spot with the overshoot guard
//     (grid.rs:486-678, heston.rs:1491-1512).
// Used only by tests and the benchmark as the judge; it is never on a product path.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <limits>
#include <vector>

#include "../include/kgpu.h"
#include "oracle_core.h"

namespace {

using kor::log_ratio;
using kor::midpoint;

constexpr double kEps = std::numeric_limits<double>::epsilon();

// scaled_cash (numerics.rs:175-186)
double scaled_cash(double amount, double exponent) {
    if (amount == 0.0) return 0.0;
    const double discount = std::exp(exponent);
    const double value = amount * discount;
    if (std::isnormal(discount) && std::isnormal(value)) return value;
    return std::exp(std::log(amount) + exponent);
}

struct Heston {
    double r, q, v0, kappa, theta, xi, rho;
};

// integrated_variance (analytic/heston.rs:436-468)
double integrated_variance(const Heston& m, double t) {
    const double x = m.kappa * t;
    if (x < 0.01) {
        double term = 0.5, sum = term;
        for (int n = 3; n <= 12; ++n) {
            term *= -x / double(n);
            sum += term;
        }
        const double transient = t * (1.0 - x * sum);
        const double growth_time = t * (t * sum);
        return m.v0 * transient + m.kappa * m.theta * growth_time;
    }
    const double complement = 1.0 + std::expm1(-x) / x;
    const double transient = -std::expm1(-x) / m.kappa;
    return m.v0 * transient + m.theta * (complement * t);
}

// variance_at (heston.rs:405-417)
double variance_at(const Heston& m, double t) {
    const double x = m.kappa * t;
    const double rise = -std::expm1(-x);
    return m.v0 * std::exp(-x) + m.theta * rise;
}

// spot_floor (grid.rs:80-86)
double spot_floor(double spot, double level, double width) {
    const double margin = std::max(width, 1e-3);
    const double wings = scaled_cash(level, -margin);
    const double query = scaled_cash(spot, -0.25 * margin);
    return std::max(std::min(wings, query), 4.9406564584124654e-324);
}

double payoff_value(double sign, double strike, double s) { return std::max(sign * (s - strike), 0.0); }

// Log-spot stencil (LogStencil / PreparedLogStencil, grid.rs:104-200).
struct Stencil {
    double left, right, down, up;
    Stencil(double l, double r) : left(l), right(r), down(-std::expm1(-l)), up(std::expm1(r)) {}
    // [lower, diagonal, upper] of the spot generator with discount `rate`.
    void coefficients(double rate, double carry, double variance, double out[3]) const {
        const double up_slope = up / right;
        const double difference = up_slope - down / left;
        double a, c;
        if (difference > 8.0 * kEps && std::isfinite(up)) {
            // The prepared form: weights divided once per node.
            const double scale = 1.0 / (difference * left);
            const double variance_weight = 0.5 * up_slope * scale;
            const double carry_weight = (1.0 - up_slope) * scale;
            const double first = variance_weight * variance + carry_weight * carry;
            a = std::max(std::max(first, -carry * (1.0 / down)), 0.0);
            c = std::max((a * down + carry) * (1.0 / up), 0.0);
        } else {
            const double drift = carry - 0.5 * variance;
            const double v = std::max(variance, std::max(drift * right, -drift * left));
            const double width = left + right;
            a = (v - drift * right) / width / left;
            c = (v + drift * left) / width / right;
        }
        out[0] = a;
        out[1] = -a - c - rate;
        out[2] = c;
    }
};

// SpatialGrid (grid.rs:222-336, 385-480): log coordinates relative to `reference`.
struct SpatialGrid {
    double lower = 0, upper = 0, spacing = 0, reference = 0;
    int count = 0;
    std::vector<double> nodes, spots;
    std::vector<Stencil> stencils;

    double coordinate(double asset) const { return log_ratio(asset, reference); }
    double asset_of_coordinate(double x) const {
        if (std::fabs(x) < 0.5) return std::fma(reference, std::expm1(x), reference);
        return scaled_cash(reference, x);
    }
    bool uniform() const { return stencils.size() == 1; }

    void set_nodes(std::vector<double> n, const std::vector<std::pair<double, double>>& anchors, bool is_uniform) {
        std::vector<double> s;
        s.push_back(lower);
        for (size_t i = 1; i + 1 < n.size(); ++i) {
            double spot = asset_of_coordinate(n[i]);
            for (const auto& a : anchors)
                if (a.first == n[i]) spot = a.second;
            s.push_back(spot);
        }
        s.push_back(upper);
        stencils.clear();
        if (is_uniform) {
            stencils.emplace_back(spacing, spacing);
        } else {
            for (size_t i = 0; i + 2 < n.size(); ++i) stencils.emplace_back(n[i + 1] - n[i], n[i + 2] - n[i + 1]);
        }
        count = int(n.size()) - 1;
        nodes = std::move(n);
        spots = std::move(s);
    }

    void init(int c, double lo, double hi, double anchor) {
        lower = lo;
        upper = hi;
        reference = std::min(std::max(anchor, lo), hi);
        const double low = log_ratio(lo, reference), high = log_ratio(hi, reference);
        spacing = (high - low) / double(c);
        count = c;
        std::vector<double> n;
        for (int i = 0; i < c; ++i) n.push_back(low + spacing * double(i));
        n.push_back(high);
        set_nodes(std::move(n), {}, true);
    }

    // concentrate_levels (grid.rs:680-781): sinh clustering of nodes at the levels.
    void concentrate(std::vector<double> levels, double scale) {
        std::vector<double> kept;
        for (double l : levels)
            if (l > lower && l < upper) kept.push_back(l);
        std::sort(kept.begin(), kept.end());
        kept.erase(std::unique(kept.begin(), kept.end()), kept.end());
        std::vector<std::pair<double, double>> anchors;
        for (double spot : kept) anchors.emplace_back(coordinate(spot), spot);
        std::vector<double> xs;
        for (const auto& a : anchors) xs.push_back(a.first);
        const double lo = nodes[0], hi = nodes[count];
        const double gap = scale * std::asinh((hi - lo) / scale) / double(count);
        double previous = lo;
        std::vector<double> retained;
        for (double l : xs) {
            if (l == lo || l == hi) {
                retained.push_back(l);
            } else if (l - previous < gap || hi - l < gap) {
                continue;
            } else {
                previous = l;
                retained.push_back(l);
            }
        }
        if (retained.empty()) return;
        struct Segment {
            double a, b;
            bool from_left;
            int steps;
            double remainder;
        };
        std::vector<Segment> segments;
        if (retained[0] > lo) segments.push_back({lo, retained[0], false, 1, 0.0});
        for (size_t i = 0; i + 1 < retained.size(); ++i) {
            const double middle = midpoint(retained[i], retained[i + 1]);
            segments.push_back({retained[i], middle, true, 1, 0.0});
            segments.push_back({middle, retained[i + 1], false, 1, 0.0});
        }
        if (retained.back() < hi) segments.push_back({retained.back(), hi, true, 1, 0.0});
        if (int(segments.size()) > count) return;
        auto width = [&](double a, double b) { return std::asinh((b - a) / scale); };
        double total = 0.0;
        for (const auto& s : segments) total += width(s.a, s.b);
        const int available = count - int(segments.size());
        int allocated = 0;
        for (auto& s : segments) {
            const double c = double(available) * width(s.a, s.b) / total;
            s.steps += int(c);
            s.remainder = c - std::floor(c);
            allocated += int(c);
        }
        for (int k = allocated; k < available; ++k) {
            size_t best = 0;
            for (size_t i = 1; i < segments.size(); ++i)
                if (segments[i].remainder > segments[best].remainder) best = i;
            segments[best].steps += 1;
            segments[best].remainder = -1.0;
        }
        double sp = total / double(count);
        for (const auto& s : segments)
            if (s.steps > 1) sp = std::min(sp, width(s.a, s.b) / (double(s.steps) - 0.5));
        std::vector<double> n{lo};
        for (const auto& s : segments) {
            for (int i = 1; i <= s.steps; ++i) {
                const double x = sp * double(s.from_left ? i : s.steps - i);
                double value;
                if (i == s.steps) value = s.b;
                else if (s.from_left) value = s.a + scale * std::sinh(x);
                else value = s.b - scale * std::sinh(x);
                if (value > n.back()) n.push_back(value);
            }
        }
        set_nodes(std::move(n), anchors, false);
    }

    const Stencil& stencil(int index) const { return stencils[uniform() ? 0 : index - 1]; }
    double cell_width(int index) const { return (nodes[index + 1] - nodes[index]) / spacing; }

    // locate (grid.rs:444-459)
    void locate(double spot, int* index, double* weight) const {
        int i = int(std::upper_bound(spots.begin(), spots.end(), spot) - spots.begin()) - 1;
        i = std::max(0, std::min(i, count - 1));
        double w;
        if (spot == spots[i + 1]) w = 1.0;
        else if (spot == spots[i]) w = 0.0;
        else w = (coordinate(spot) - nodes[i]) / (nodes[i + 1] - nodes[i]);
        *index = i;
        *weight = w;
    }

    // Cell average of a kinked payoff (project_payoff, grid.rs:14-78): two-point Gauss
    // rule on the pieces of the node's dual cell split at the kink.
    double project(double kink, int index, double sign, double strike) const {
        const double center = nodes[index];
        if (index == 0 || index == count) return payoff_value(sign, strike, spots[index]);
        const double lo = midpoint(nodes[index - 1], center), hi = midpoint(center, nodes[index + 1]);
        const double b = coordinate(kink);
        if (!(kink > 0.0) || !(b > lo && b < hi)) return payoff_value(sign, strike, spots[index]);
        std::vector<double> points{b, lo, center, hi};
        std::sort(points.begin(), points.end());
        points.erase(std::unique(points.begin(), points.end()), points.end());
        auto value = [&](double x) {
            return x == center ? payoff_value(sign, strike, spots[index])
                               : payoff_value(sign, strike, asset_of_coordinate(x));
        };
        double result = 0.0;
        for (size_t i = 0; i + 1 < points.size(); ++i) {
            const double middle = midpoint(points[i], points[i + 1]);
            const double radius = (points[i + 1] - points[i]) / (2.0 * std::sqrt(3.0));
            const double low = value(middle - radius), high = value(middle + radius);
            result += (points[i + 1] - points[i]) / (hi - lo) * midpoint(low, high);
        }
        return result;
    }

    // Natural-ish cubic spline curvature in normalised log coordinates (grid.rs:513-560).
    std::vector<double> curvature(const std::vector<double>& values) const {
        std::vector<double> curv(values.size(), 0.0), factors(values.size(), 0.0);
        auto end_ratio = [&](int outer, int inner, double* out) {
            const double ratio = cell_width(outer) / cell_width(inner);
            if (ratio >= 0.25 && ratio <= 4.0) {
                *out = ratio;
                return true;
            }
            return false;
        };
        double first_ratio = 0, last_ratio = 0;
        const bool has_first = end_ratio(0, 1, &first_ratio);
        const bool has_last = end_ratio(count - 1, count - 2, &last_ratio);
        for (int node = 1; node < count; ++node) {
            const double left = cell_width(node - 1), right = cell_width(node);
            const double total = left + right;
            double a = left / total, c = right / total, diagonal = 2.0;
            if (has_first && node == 1) {
                diagonal += a * (1.0 + first_ratio);
                c -= a * first_ratio;
                a = 0.0;
            }
            if (has_last && node == count - 1) {
                diagonal += c * (1.0 + last_ratio);
                a -= c * last_ratio;
                c = 0.0;
            }
            diagonal -= a * factors[node - 1];
            factors[node] = c / diagonal;
            curv[node] = (6.0 * (((values[node + 1] - values[node]) / right - (values[node] - values[node - 1]) / left) /
                                 total) -
                          a * curv[node - 1]) /
                         diagonal;
        }
        for (int node = count - 1; node >= 1; --node) curv[node] -= factors[node] * curv[node + 1];
        if (has_first) curv[0] = curv[1] + first_ratio * (curv[1] - curv[2]);
        if (has_last) curv[count] = curv[count - 1] + last_ratio * (curv[count - 1] - curv[count - 2]);
        return curv;
    }

    // Price read-out of sample_log (grid.rs:582-678), without the derivative outputs.
    double sample(const std::vector<double>& values, double spot) const {
        const std::vector<double> curv = curvature(values);
        double global_min = values[0], global_max = values[0];
        for (double v : values) {
            global_min = std::min(global_min, v);
            global_max = std::max(global_max, v);
        }
        int index;
        double weight;
        locate(spot, &index, &weight);
        if (index > 0 && index + 2 <= count) {
            auto slope = [&](int i) { return (values[i + 1] - values[i]) / (spots[i + 1] - spots[i]); };
            const double here = slope(index);
            const double tolerance = 5e-9 * std::fabs(here);
            if (std::isfinite(here) && std::fabs(slope(index - 1) - here) <= tolerance &&
                std::fabs(slope(index + 1) - here) <= tolerance)
                return std::fma(here, spot - spots[index], values[index]);
        }
        const double h = cell_width(index);
        const double left = 1.0 - weight;
        const double linear = values[index] + weight * (values[index + 1] - values[index]);
        const double correction =
            ((left * left * left - left) * curv[index] + (weight * weight * weight - weight) * curv[index + 1]) / 6.0;
        const double interpolated = linear + correction * h * h;
        const double first_control =
            values[index] + (values[index + 1] - values[index]) / 3.0 - (2.0 * curv[index] + curv[index + 1]) * h * h / 18.0;
        const double second_control = values[index] + 2.0 * (values[index + 1] - values[index]) / 3.0 -
                                      (curv[index] + 2.0 * curv[index + 1]) * h * h / 18.0;
        const double minimum = std::min(values[index], values[index + 1]);
        const double maximum = std::max(values[index], values[index + 1]);
        const bool overshoot = uniform() ? (interpolated < minimum || interpolated > maximum)
                                         : (std::min(first_control, second_control) < minimum ||
                                            std::max(first_control, second_control) > maximum);
        if (overshoot) {
            const double slope = (values[index + 1] - values[index]) / h;
            const double before = index > 0 ? (values[index] - values[index - 1]) / cell_width(index - 1) : slope;
            const double after =
                index + 2 < int(values.size()) ? (values[index + 2] - values[index + 1]) / cell_width(index + 1) : slope;
            const double first = slope - h * (2.0 * curv[index] + curv[index + 1]) / 6.0;
            const double last = slope + h * (curv[index] + 2.0 * curv[index + 1]) / 6.0;
            const bool maximum_turn = before > 0.0 && after < 0.0 && curv[index] <= 0.0 && curv[index + 1] <= 0.0 &&
                                      first <= before && last >= after;
            const bool minimum_turn = before < 0.0 && after > 0.0 && curv[index] >= 0.0 && curv[index + 1] >= 0.0 &&
                                      first >= before && last <= after;
            if (!maximum_turn && !minimum_turn) {
                if (uniform()) return std::min(std::max(interpolated, minimum), maximum);
                if (std::min(first_control, second_control) < global_min ||
                    std::max(first_control, second_control) > global_max)
                    return linear;
            }
        }
        if (weight == 0.0) return values[index];
        if (weight == 1.0) return values[index + 1];
        return interpolated;
    }
};

// directional (heston.rs:1571-1586): upwinded generator row on a nonuniform axis.
void directional(const std::vector<double>& n, size_t i, double diffusion, double drift, double discount,
                 double out[3]) {
    if (i == 0) {
        const double c = drift / (n[1] - n[0]);
        out[0] = 0.0;
        out[1] = -c - discount;
        out[2] = c;
        return;
    }
    const double left = n[i] - n[i - 1], right = n[i + 1] - n[i], span = left + right;
    double a = (2.0 * diffusion - drift * right) / (left * span);
    double c = (2.0 * diffusion + drift * left) / (right * span);
    if (a < 0.0 || c < 0.0) {
        a = 2.0 * diffusion / (left * span) + std::max(-drift, 0.0) / left;
        c = 2.0 * diffusion / (right * span) + std::max(drift, 0.0) / right;
    }
    out[0] = a;
    out[1] = -a - c - discount;
    out[2] = c;
}

// derivative (heston.rs:1588-1596): central first-derivative weights.
void derivative(const std::vector<double>& n, size_t i, double out[3]) {
    const double left = n[i] - n[i - 1], right = n[i + 1] - n[i];
    out[0] = -right / (left * (left + right));
    out[1] = (right - left) / (left * right);
    out[2] = left / (right * (left + right));
}

// Asset-edge rule of ExerciseBoundaries for flat curves (deterministic.rs:386-531).
struct EdgeRule {
    enum Kind { Zero, Immediate, Expiry, Scan } kind;
};

double discounted_intrinsic(double sign, double strike, double spot, double dividend_log, double risk_log) {
    const double moneyness = log_ratio(spot, strike) + (dividend_log - risk_log);
    if (sign * moneyness <= 0.0) return 0.0;
    if (sign > 0.0) return scaled_cash(spot, dividend_log + std::log(-std::expm1(-moneyness)));
    return scaled_cash(strike, risk_log + std::log(-std::expm1(moneyness)));
}

}  // namespace

// Heston ADI price of a vanilla option; `sign` +1 call, -1 put.  Returns NaN for an
// unusable grid.  Grid sizes are interval counts (defaults 400 x 100 x 400).
extern "C" double kor_heston_adi_american(const kgpu_model* model, double strike, double sign, double expiry,
                                          int asset_steps, int variance_steps, int time_steps, int american) {
    const double nan = std::numeric_limits<double>::quiet_NaN();
    if (!model || model->kind != KGPU_MODEL_HESTON || !(strike > 0.0) || !(expiry > 0.0) || asset_steps < 3 ||
        variance_steps < 3 || time_steps < 1 || !(model->xi > 0.0))
        return nan;
    const Heston m{model->rate, model->dividend, model->v0, model->kappa, model->theta, model->xi, model->rho};
    const double spot0 = model->spot;
    const double T = expiry;
    // Scaled units (heston.rs:712-722).
    const double scale = std::max(strike, spot0);
    const double K = strike / scale;
    const double minimum_spot = spot0 / scale;
    const double integrated = integrated_variance(m, T);
    // Flat curves: the only curve knot is expiry (curve.rs:62-64).
    const double carry_T = (m.r - m.q) * T;
    const double drift = std::max(0.0, carry_T), lower_drift = std::max(0.0, -carry_T);
    const double upper = std::max(std::exp(drift + 6.0 * std::sqrt(integrated)), 4.0);
    const double width = std::sqrt(integrated);
    const double tail_width = std::max(width, 0.35 * m.xi * T);
    const double lower = spot_floor(minimum_spot, K, lower_drift + 0.5 * integrated + 6.0 * tail_width);
    SpatialGrid asset;
    asset.init(asset_steps, lower, upper, K);
    if (width > 0.0 && width < 0.04 && std::fabs(carry_T) > 4.0 * width) return nan;  // drift band: not needed here
    const double asset_scale = width < 0.04 ? std::max(0.3 * width, kEps) : 0.06;
    asset.concentrate({K}, asset_scale);
    // Variance grid (heston.rs:905-934, 419-440).
    const double mean = std::max(m.v0, variance_at(m, T));
    const double horizon = m.kappa * T == 0.0 ? T : -std::expm1(-2.0 * m.kappa * T) / m.kappa / 2.0;
    const double spread = m.xi * std::sqrt(mean * horizon);
    const double v_upper = std::max(mean + 8.0 * spread, 0.25);
    const double v_scale = std::max(std::max(0.1 * mean, 0.05 * spread), 0.0001);
    std::vector<double> vn;
    {
        const double end = std::asinh(v_upper / v_scale);
        const double spacing = end / double(variance_steps);
        for (int i = 0; i < variance_steps; ++i) vn.push_back(v_scale * std::sinh(spacing * double(i)));
        vn.push_back(v_upper);
    }
    int valuation_row = 0;
    if (m.v0 > 0.0) {
        valuation_row = 1;
        for (int j = 2; j < int(vn.size()) - 1; ++j)
            if (std::fabs(vn[j] - m.v0) < std::fabs(vn[valuation_row] - m.v0)) valuation_row = j;
        vn[valuation_row] = m.v0;
    }
    const int nx = asset.count + 1;
    const int rows = int(vn.size());
    const int dyn = rows - 1;
    // Operators (heston.rs:1662-1719, 1725-1881).
    std::vector<std::array<double, 3>> vbase(dyn), dx(nx, {0, 0, 0}), dv(rows, {0, 0, 0});
    std::vector<double> mixed(rows, 0.0);
    for (int j = 0; j < dyn; ++j) {
        double row[3];
        directional(vn, size_t(j), 0.5 * m.xi * m.xi * vn[j], m.kappa * (m.theta - vn[j]), 0.0, row);
        vbase[j] = {row[0], row[1], row[2]};
        mixed[j] = m.rho * m.xi * vn[j];
    }
    for (int i = 1; i < nx - 1; ++i) {
        double d[3];
        derivative(asset.nodes, size_t(i), d);
        dx[i] = {d[0], d[1], d[2]};
    }
    for (int j = 1; j < rows - 1; ++j) {
        double d[3];
        derivative(vn, size_t(j), d);
        dv[j] = {d[0], d[1], d[2]};
    }
    const double rate = m.r, q = m.q;
    // Asset rows per variance row, with half the discount (heston.rs:1792-1800).
    std::vector<std::array<double, 3>> amat(size_t(rows) * nx, {0, 0, 0});
    for (int j = 0; j < dyn; ++j)
        for (int i = 1; i < nx - 1; ++i) {
            double c[3];
            asset.stencil(i).coefficients(rate, rate - q, vn[j], c);
            c[1] += rate / 2.0;
            amat[size_t(j) * nx + i] = {c[0], c[1], c[2]};
        }
    std::vector<std::array<double, 3>> vmat(rows, {0, 0, 0});
    for (int j = 0; j < dyn; ++j) vmat[j] = {vbase[j][0], vbase[j][1] - rate / 2.0, vbase[j][2]};
    // Uniform time grid (grid.rs:930-1022 with no interior events).
    const double dt = T / double(time_steps);
    const double weight = dt / 3.0;
    // Factorisations of (I - weight A_direction) (heston.rs:1840-1880, 2644-2665).
    std::vector<std::array<double, 3>> afac(size_t(dyn) * nx);
    for (int j = 0; j < dyn; ++j) {
        double prev_diag = 1.0, prev_upper = 0.0;
        for (int i = 0; i < nx; ++i) {
            const auto& row = amat[size_t(j) * nx + i];
            double mult = -weight * row[0], diag = 1.0 - weight * row[1];
            const double upp = -weight * row[2];
            if (i > 0) {
                mult /= prev_diag;
                diag -= mult * prev_upper;
            }
            if (!std::isfinite(diag) || diag == 0.0) return nan;
            afac[size_t(j) * nx + i] = {mult, diag, upp};
            prev_diag = diag;
            prev_upper = upp;
        }
    }
    std::vector<std::array<double, 3>> vfac(rows);
    for (int j = 0; j < dyn; ++j) vfac[j] = {-weight * vmat[j][0], 1.0 - weight * vmat[j][1], -weight * vmat[j][2]};
    vfac[dyn] = {-1.0, 1.0, 0.0};
    for (int j = 1; j < rows; ++j) {
        vfac[j][0] /= vfac[j - 1][1];
        vfac[j][1] -= vfac[j][0] * vfac[j - 1][2];
        if (!std::isfinite(vfac[j][1]) || vfac[j][1] == 0.0) return nan;
    }
    // Terminal values, intrinsic values and edges.
    const size_t length = size_t(rows) * nx;
    std::vector<double> values(length), intrinsic(nx), lambda(american ? length : 0, 0.0), pred(length, 0.0),
        stage(length, 0.0);
    for (int i = 0; i < nx; ++i) {
        const double t = asset.project(K, i, sign, K);
        for (int j = 0; j < rows; ++j) values[size_t(j) * nx + i] = t;
        intrinsic[i] = payoff_value(sign, K, asset.spots[i]);
    }
    // Exercise-boundary rules at both asset edges (deterministic.rs:398-433).
    EdgeRule::Kind rules[2] = {EdgeRule::Expiry, EdgeRule::Expiry};
    if (american) {
        const double c0 = std::min(0.0, carry_T), c1 = std::max(0.0, carry_T);
        double th0 = -INFINITY, th1 = INFINITY;
        if (m.r > 0.0 && m.q > 0.0) th0 = th1 = log_ratio(m.r, m.q);
        const double bounds[2] = {lower, upper};
        for (int side = 0; side < 2; ++side) {
            const double center = log_ratio(bounds[side], K);
            const double margin = 1e-10 * (1.0 + std::fabs(center) + std::fabs(c0) + std::fabs(c1));
            const double low = center - (c1 - c0) - margin, high = center + (c1 - c0) + margin;
            const bool call = sign > 0.0;
            if ((call && high < 0.0) || (!call && low > 0.0)) rules[side] = EdgeRule::Zero;
            else if ((call && low > th1) || (!call && high < th0)) rules[side] = EdgeRule::Immediate;
            else if ((call && high < th0) || (!call && low > th1)) rules[side] = EdgeRule::Expiry;
            else rules[side] = EdgeRule::Scan;
        }
    }
    auto edge_value = [&](int side, double start) {
        const double s = side == 0 ? lower : upper;
        const double tau = T - start;
        switch (rules[side]) {
            case EdgeRule::Zero: return 0.0;
            case EdgeRule::Immediate: return payoff_value(sign, K, s);
            case EdgeRule::Expiry: return discounted_intrinsic(sign, K, s, -q * tau, -rate * tau);
            case EdgeRule::Scan:
                return std::max(payoff_value(sign, K, s), discounted_intrinsic(sign, K, s, -q * tau, -rate * tau));
        }
        return 0.0;
    };
    // One explicit evaluation of (A0, A1 + A2) at variance row j (heston.rs:1900-1956).
    auto components = [&](const std::vector<double>& v, int j, int i, double* mix, double* along) {
        const double* cur = &v[size_t(j) * nx];
        const double* prev = &v[size_t(std::max(j - 1, 0)) * nx];
        const double* next = &v[size_t(j + 1) * nx];
        const auto& a = amat[size_t(j) * nx + i];
        const double asset_term = a[0] * cur[i - 1] + a[1] * cur[i] + a[2] * cur[i + 1];
        double variance_term = vmat[j][1] * cur[i];
        if (j > 0) variance_term += vmat[j][0] * prev[i];
        variance_term += vmat[j][2] * next[i];
        double mixed_term = 0.0;
        if (j > 0) {
            const double lw = dv[j][0], rw = dv[j][2];
            auto diff = [&](int k) { return lw * (prev[k] - cur[k]) + rw * (next[k] - cur[k]); };
            const double left = diff(i - 1), center = diff(i), right = diff(i + 1);
            mixed_term = mixed[j] * (dx[i][0] * (left - center) + dx[i][2] * (right - center));
        }
        *mix = mixed_term;
        *along = asset_term + variance_term;
    };
    // (I - weight A1)^-1 then (I - weight A2)^-1 on increments (heston.rs:2285-2347).
    auto solve = [&](std::vector<double>& v, double e0, double e1) {
        for (int j = 0; j < dyn; ++j) {
            double* row = &v[size_t(j) * nx];
            const auto* f = &afac[size_t(j) * nx];
            double previous = e0;
            for (int i = 1; i < nx - 1; ++i) {
                row[i] -= f[i][0] * previous;
                previous = row[i];
            }
            double next = e1;
            for (int i = nx - 2; i >= 1; --i) {
                row[i] = (row[i] - f[i][2] * next) / f[i][1];
                next = row[i];
            }
            row[0] = e0;
            row[nx - 1] = e1;
        }
        for (int j = 1; j < rows; ++j) {
            double* row = &v[size_t(j) * nx];
            const double* prior = &v[size_t(j - 1) * nx];
            if (j < dyn)
                for (int i = 0; i < nx; ++i) row[i] -= vfac[j][0] * prior[i];
            else
                for (int i = 0; i < nx; ++i) row[i] = -vfac[j][0] * prior[i];
        }
        for (int j = rows - 1; j >= 0; --j) {
            double* row = &v[size_t(j) * nx];
            const double inverse = 1.0 / vfac[j][1];
            const bool reciprocal = std::isnormal(inverse);
            if (j + 1 < rows) {
                const double* other = &v[size_t(j + 1) * nx];
                for (int i = 0; i < nx; ++i) {
                    const double x = row[i] - vfac[j][2] * other[i];
                    row[i] = reciprocal ? x * inverse : x / vfac[j][1];
                }
            } else {
                for (int i = 0; i < nx; ++i) row[i] = reciprocal ? row[i] * inverse : row[i] / vfac[j][1];
            }
        }
        for (int j = 0; j < rows; ++j) {
            v[size_t(j) * nx] = e0;
            v[size_t(j) * nx + nx - 1] = e1;
        }
        std::copy(v.begin() + size_t(rows - 2) * nx, v.begin() + size_t(rows - 1) * nx, v.begin() + size_t(rows - 1) * nx);
    };
    for (int step = time_steps - 1; step >= 0; --step) {
        const double a_time = step == 0 ? 0.0 : T * double(step) / double(time_steps);
        const double e0 = edge_value(0, a_time), e1 = edge_value(1, a_time);
        const double d0 = e0 - values[0], d1 = e1 - values[nx - 1];
        // Y0 = dt (A V + lambda) (predict, heston.rs:1958-2003).
        for (int j = 0; j < dyn; ++j)
            for (int i = 1; i < nx - 1; ++i) {
                double mix, along;
                components(values, j, i, &mix, &along);
                const size_t k = size_t(j) * nx + i;
                const double correction = american ? lambda[k] : 0.0;
                const double value = dt * (mix + along + correction);
                pred[k] = value;
                stage[k] = value;
            }
        solve(stage, d0, d1);
        // Ytilde0 = Y0 + dt (A0 D2 / 2 + (A1 + A2) D2 / 6) (correct, heston.rs:2005-2041).
        for (int j = 0; j < dyn; ++j)
            for (int i = 1; i < nx - 1; ++i) {
                double mix, along;
                components(stage, j, i, &mix, &along);
                pred[size_t(j) * nx + i] += dt * (0.5 * mix + along / 6.0);
            }
        solve(pred, d0, d1);
        if (american) {
            // Ikonen-Toivanen splitting (exercise, heston.rs:2043-2103).
            for (int j = 0; j < rows; ++j) {
                for (int i = 0; i < nx; ++i) {
                    const size_t k = size_t(j) * nx + i;
                    const double raw = values[k] + pred[k];
                    pred[k] = std::max(raw - dt * lambda[k], intrinsic[i]);
                    lambda[k] = std::max(lambda[k] + (intrinsic[i] - raw) / dt, 0.0);
                }
                pred[size_t(j) * nx] = e0;
                pred[size_t(j) * nx + nx - 1] = e1;
            }
        } else {
            for (size_t k = 0; k < length; ++k) pred[k] += values[k];
            for (int j = 0; j < rows; ++j) {
                pred[size_t(j) * nx] = e0;
                pred[size_t(j) * nx + nx - 1] = e1;
            }
        }
        std::copy(pred.begin() + size_t(rows - 2) * nx, pred.begin() + size_t(rows - 1) * nx,
                  pred.begin() + size_t(rows - 1) * nx);
        std::swap(values, pred);
        for (double x : values)
            if (!std::isfinite(x)) return nan;
    }
    // Read-out on the valuation row (grid_price, heston.rs:1491-1512).
    const std::vector<double> row(values.begin() + size_t(valuation_row) * nx,
                                  values.begin() + size_t(valuation_row + 1) * nx);
    const double s = spot0 / scale;
    double price = asset.sample(row, s);
    if (american) {
        const double exercise = payoff_value(sign, K, s);
        int index;
        double w;
        asset.locate(s, &index, &w);
        const bool exercised = row[index] == payoff_value(sign, K, asset.spots[index]) &&
                               row[index + 1] == payoff_value(sign, K, asset.spots[index + 1]);
        price = exercised ? exercise : std::max(price, exercise);
    }
    return scale * price;
}
