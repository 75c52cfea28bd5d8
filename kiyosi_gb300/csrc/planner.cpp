// Host planner of a book of autocallable notes on one shared daily grid (no GPU).
//
// The planning half of MonteCarloAutocallableEngine::price_many_on_shared_grid
// (crates/kiyosi/src/engines/monte_carlo/autocallable/portfolio.rs), for BSM books:
//   * which notes join a shared daily grid: daily knock-in monitoring that still matters,
//     cash events on monitoring dates or expiry (DailyGrids::prepare, portfolio.rs:74-185),
//     each note's plan being prepare_sample_on_grid's (autocallable.rs:293-430) without
//     the Brownian-bridge plan;
//   * the groups of notes of one daily grid (same_daily_grid, portfolio.rs:872-901);
//   * the coupon families of three or more notes differing only in their coupon, priced
//     from the lowest- and highest-coupon members (price_coupon_families, 570-667);
//   * each group's interval plan, bridging runs of at least eight daily steps between
//     action dates (SharedEvents::new, 903-1047), and one bridged lane contract per
//     simulated note, laid out for the path-major kernel.
// A note the reference would reject (missing history, a non-finite plan), or that needs
// no sampling, is left to the scalar engine's planner, which reports or values it.
//
// Layout (one kgpu_book per group): lanes of one maturity and one set of event steps
// have the same steps, flags and bridge weights -- prefixes of the group's longest grid
// -- so they share one segment of the step arrays; every lane's intervals are a prefix
// of the group's interval list.  A 4,096-note book on one 504-step grid is then a few
// segments instead of one 25 KB copy per lane.  Each lane's contract and events are its
// own.
//
// Floating point follows the reference's order of operations with contraction off
// (the build passes -ffp-contract=off), so plans equal the Python restatement's
// (kiyosi_gb300/portfolio.py, kiyosi_gb300/plans.py) bit for bit.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <new>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "../../include/kgpu.h"

namespace kgpu {
void set_thread_error(const char* message);
}

struct kgpu_shared_plan {
    struct Group {
        std::vector<kgpu_contract> contracts;
        std::vector<kgpu_step> steps;
        std::vector<uint8_t> flags;
        std::vector<kgpu_bridge_daily> daily;
        std::vector<kgpu_event> events;
        std::vector<kgpu_bridge_interval> intervals;
    };
    struct Strip {
        std::vector<int32_t> members;  // book indices
        int32_t low = 0, high = 0;     // book indices
        double width = 0.0;
    };
    int32_t note_count = 0;
    std::vector<int32_t> note_group;
    std::vector<int32_t> group_first_lane;
    std::vector<int32_t> lane_note;
    std::vector<uint8_t> lane_fp32;
    std::vector<Group> groups;
    std::vector<kgpu_book> group_books;
    std::vector<int32_t> group_status;
    std::vector<std::string> message_text;
    std::vector<const char*> group_message;
    std::vector<Strip> strips;
    std::vector<double> coupon;       // portfolio coupon per note
    std::vector<uint8_t> simulated;   // per note
};

namespace {

constexpr double kSmallestNormal = 2.2250738585072014e-308;
constexpr double kInf = std::numeric_limits<double>::infinity();
constexpr double kNan = std::numeric_limits<double>::quiet_NaN();

bool is_normal(double x) { return std::isfinite(x) && std::fabs(x) >= kSmallestNormal; }

// A step of the planner that the reference (or its Python restatement) would refuse:
// the note goes to the scalar engine's planner, which raises the matching error.
struct Defer {};

// exp that refuses an overflow from a finite argument (Python's math.exp raises there).
double checked_exp(double x) {
    const double r = std::exp(x);
    if (std::isinf(r) && std::isfinite(x)) throw Defer{};
    return r;
}

double checked_log(double x) {
    if (!(x > 0.0) && !std::isnan(x)) throw Defer{};  // a domain error in the restatement
    return std::log(x);
}

double safe_log(double x) { return x == 0.0 ? -kInf : checked_log(x); }

// numerics.rs:80-92
double log_ratio(double numerator, double denominator) {
    const double relative = (numerator - denominator) / denominator;
    if (std::fabs(relative) < 0.5) return std::log1p(relative);
    const double ratio = numerator / denominator;
    if (ratio != 0.0 && std::isfinite(ratio) && std::fabs(ratio) >= kSmallestNormal) return checked_log(ratio);
    return safe_log(numerator) - safe_log(denominator);
}

// safe_log_returns (monte_carlo.rs:2139-2145)
void safe_log_returns(double spot, double* low, double* high) {
    const double log_spot = std::log(spot);
    const double lo = std::log(kSmallestNormal) + 1.0;
    const double hi = std::log(std::numeric_limits<double>::max()) - 1.0;
    *low = std::max(lo, lo - log_spot);
    *high = std::min(hi, hi - log_spot);
}

// numerics.rs:226-238
double discounted_product(double scale, double weight, double log_discount) {
    const double value = scale * weight;
    const double discount = log_discount < 709.0 ? std::exp(log_discount) : kInf;
    if (scale == 0.0 || weight == 0.0) return 0.0;
    if (is_normal(discount) && is_normal(value)) return value * discount;
    return std::copysign(checked_exp(checked_log(scale) + checked_log(std::fabs(weight)) + log_discount), weight);
}

// Python's max(a, b) / min(a, b): the first argument unless the second compares beyond it.
double py_max(double a, double b) { return b > a ? b : a; }
double py_min(double a, double b) { return b < a ? b : a; }

// One note and its table ranges (AutocallableNote, instruments/autocallable.rs).
struct Note {
    const kgpu_note* n = nullptr;
    const kgpu_note_observation* obs = nullptr;
    int obs_count = 0;
    const double* mon = nullptr;
    int mon_count = 0;

    bool has_ki() const { return (n->flags & KGPU_NOTE_KNOCK_IN) != 0; }
    bool monitored() const { return (n->flags & KGPU_NOTE_MONITORING) != 0; }
    bool fixed() const { return (n->flags & KGPU_NOTE_FIXED_COUPON) != 0; }
    bool daily_knock_in() const { return has_ki() && monitored(); }
    static bool has_ko(const kgpu_note_observation& o) { return (o.flags & KGPU_OBSERVATION_KNOCK_OUT) != 0; }
    static bool has_cb(const kgpu_note_observation& o) { return (o.flags & KGPU_OBSERVATION_COUPON_BARRIER) != 0; }

    // autocallable.rs:1415-1418
    double rebate_payment(double time) const { return n->rebate_rate + n->annual_rebate_rate * (time - n->effective_time); }
    // autocallable.rs:1419-1424
    double knock_out_payment(const kgpu_note_observation& o) const {
        return n->principal + rebate_payment(o.time) + o.coupon_rate * (o.time - n->effective_time);
    }
    // autocallable.rs:1396-1414
    double terminal(double spot, bool knocked_in) const {
        const double base = n->principal + rebate_payment(n->expiry);
        double coupon;
        if (knocked_in) {
            if (!fixed()) {
                const double clamped = py_min(py_max(spot, n->lower_strike), n->upper_strike);
                return base + (clamped - n->upper_strike) / n->initial_spot;
            }
            coupon = n->fixed_knock_in_coupon;
        } else {
            coupon = n->maturity_coupon_rate;
        }
        return base + coupon * (n->expiry - n->effective_time);
    }
    // Monitoring times are strictly increasing (checked when the plan is created).
    bool monitors(double time) const { return mon_count > 0 && std::binary_search(mon, mon + mon_count, time); }
    // autocallable.rs:1075-1080
    bool observes_knock_in(double time) const {
        if (!has_ki()) return false;
        if (monitored()) return monitors(time);
        return time == n->expiry;
    }
    // autocallable.rs:1652-1654 (strict)
    bool below_knock_in(double spot) const { return has_ki() && spot < n->knock_in_level; }
    // autocallable.rs:1164-1174
    double observation_coupon(const kgpu_note_observation* o, double spot) const {
        if (o && has_cb(*o) && spot >= o->coupon_barrier_level) return n->period_coupon;
        return 0.0;
    }
    // autocallable.rs:1323-1332
    bool knock_in_affects_payoff() const {
        if (!has_ki()) return false;
        if (fixed()) return n->fixed_knock_in_coupon != n->maturity_coupon_rate;
        return n->lower_strike != n->upper_strike || n->maturity_coupon_rate != 0.0;
    }
    bool phoenix() const {
        for (int k = 0; k < obs_count; ++k)
            if (has_cb(obs[k])) return true;
        return false;
    }
    // AutocallableNote::portfolio_coupon (autocallable.rs:1182-1186)
    double portfolio_coupon() const { return phoenix() ? n->period_coupon : n->maturity_coupon_rate; }
};

// AutocallableNote::prior (autocallable.rs:1320-1369): false where the reference refuses
// the recorded history.
bool prior_ok(const Note& note) {
    const kgpu_note& n = *note.n;
    bool have_first = false;
    double first_out = 0.0;
    for (int k = 0; k < note.obs_count && !have_first; ++k)
        if (Note::has_ko(note.obs[k])) {
            first_out = note.obs[k].time;
            have_first = true;
        }
    if (!have_first && note.obs_count > 0) {
        first_out = note.obs[0].time;
        have_first = true;
    }
    const bool had_out = have_first && first_out < 0.0;
    bool had_in = false;
    if (note.daily_knock_in() && n.effective_time < 0.0)
        for (int k = 0; k < note.mon_count; ++k)
            if (n.effective_time <= note.mon[k] && note.mon[k] < 0.0) had_in = true;
    const int state = n.barrier_state;
    if (state == KGPU_STATE_UNKNOWN && (had_out || had_in)) return false;
    if (state == KGPU_STATE_KNOCKED_OUT && !had_out) return false;
    if (state == KGPU_STATE_KNOCKED_IN && !had_in) return false;
    return true;
}

struct Initial {
    bool knocked_in = false;
    bool settles = false;  // a settlement at valuation: no sampling
    double coupon = 0.0;
};

// pricing::initial (instruments/autocallable/pricing.rs:12-49) at valuation.  The
// settlement's amount is the scalar planner's business; only its presence matters here.
Initial initial_state(const Note& note, double spot) {
    const kgpu_note& n = *note.n;
    Initial s;
    if (n.barrier_state == KGPU_STATE_KNOCKED_OUT) {
        s.settles = true;
        return s;
    }
    s.knocked_in = n.barrier_state == KGPU_STATE_KNOCKED_IN;
    if (note.daily_knock_in() && note.monitors(0.0)) s.knocked_in = s.knocked_in || note.below_knock_in(spot);
    const kgpu_note_observation* current = nullptr;
    for (int k = 0; k < note.obs_count && !current; ++k)
        if (note.obs[k].time == 0.0) current = &note.obs[k];
    s.coupon = note.observation_coupon(current, spot);
    if (n.expiry == 0.0)
        s.settles = true;
    else if (current && Note::has_ko(*current) && spot >= current->knock_out_level)
        s.settles = true;
    return s;
}

// pricing::fixed_value_at (instruments/autocallable/pricing.rs:137-193): whether no
// remaining path can change the note's value (then the scalar planner values it).
bool fixed_value(const Note& note, double spot, double rate, bool knocked_in) {
    const kgpu_note& n = *note.n;
    bool pending;
    if (note.daily_knock_in()) {
        pending = false;
        if (n.expiry > 0.0)
            for (int k = 0; k < note.mon_count && !pending; ++k)
                if (0.0 < note.mon[k] && note.mon[k] <= n.expiry) pending = true;
    } else {
        pending = note.has_ki() && n.expiry > 0.0;
    }
    if (knocked_in || pending) {
        if (!note.fixed() && note.has_ki()) {
            if (n.lower_strike != n.upper_strike || (!knocked_in && n.maturity_coupon_rate != 0.0)) return false;
        } else if (!knocked_in && note.knock_in_affects_payoff()) {
            return false;
        }
    }
    auto discount = [&](double t) { return checked_exp(-rate * t); };
    const double value = note.terminal(spot, knocked_in) * discount(n.expiry);
    if (!std::isfinite(value)) return false;
    double coupons = 0.0;
    for (int k = note.obs_count - 1; k >= 0; --k) {
        const kgpu_note_observation& o = note.obs[k];
        if (!(o.time > 0.0)) break;
        const double d = discount(o.time);
        if (!is_normal(d) || (Note::has_ko(o) && note.knock_out_payment(o) * d != value + coupons)) return false;
        if (Note::has_cb(o)) {
            if (n.period_coupon != 0.0 && o.coupon_barrier_level != 0.0) return false;
            coupons += n.period_coupon * d;
            if (!std::isfinite(coupons)) return false;
        }
    }
    return is_normal(discount(n.expiry));
}

// One note's merged grid of future event dates, daily knock-in dates and expiry
// (future_event_times, instruments/autocallable/pricing.rs:70-106) under BSM: the step
// records, knock-in flags and excursion.  Notes with one schedule share it.
struct Grid {
    std::vector<double> times;
    std::vector<kgpu_step> steps;
    std::vector<uint8_t> knock_in;
};

// CashEvent::new and discounted_payment (autocallable.rs:532-562)
kgpu_event cash_event(const Note& note, const kgpu_note_observation& o, double spot, double rate, int step) {
    kgpu_event e{};
    const bool has_ko = Note::has_ko(o);
    e.knock_out = has_ko ? log_ratio(o.knock_out_level, spot) : 0.0;
    e.coupon_barrier = log_ratio(Note::has_cb(o) ? o.coupon_barrier_level : 0.0, spot);
    const double period_coupon = Note::has_cb(o) ? note.n->period_coupon : 0.0;
    const double redemption = has_ko ? note.knock_out_payment(o) : 0.0;
    const double log_discount = -rate * o.time;
    const double discount = log_discount < 709.0 ? std::exp(log_discount) : kInf;
    const bool plain = std::isfinite(discount) && discount >= kSmallestNormal;
    for (int outcome = 0; outcome < 4; ++outcome) {
        const bool coupon_due = (outcome & 1) != 0, knocked_out = (outcome >> 1) != 0;
        const double coupon = coupon_due ? period_coupon : 0.0;
        const double amount = knocked_out ? redemption + coupon : coupon;
        if (amount == 0.0)
            e.payment[outcome] = 0.0;
        else if (plain && std::isfinite(amount) && std::fabs(amount) >= kSmallestNormal)
            e.payment[outcome] = amount * discount;
        else
            e.payment[outcome] = discounted_product(1.0, amount, log_discount);
    }
    e.has_knock_out = has_ko ? 1 : 0;
    e.step = step;
    return e;
}

struct Lane {
    int note = 0;
    bool sparse = false;
    bool maturity_on_grid = false;
    const Grid* grid = nullptr;   // steps and knock-in flags (shared)
    int steps = 0;                // maturity + 1
    kgpu_contract contract{};
    std::vector<kgpu_event> events;
};

struct Model {
    double spot, rate, dividend, sigma;
};

// transition (engines/monte_carlo.rs:2123-2137) over a grid; Defer on a non-finite value.
void grid_steps(const Model& m, Grid& g) {
    const size_t n = g.times.size();
    g.steps.resize(n);
    double previous = 0.0;
    for (size_t i = 0; i < n; ++i) {
        const double t = g.times[i];
        const double dt = t - previous;
        const double drift = (m.rate - m.dividend - 0.5 * m.sigma * m.sigma) * dt;
        const double diffusion = m.sigma * std::sqrt(dt);
        const double log_discount = -m.rate * t;
        if (!(std::isfinite(drift) && std::isfinite(diffusion) && std::isfinite(log_discount))) throw Defer{};
        g.steps[i] = kgpu_step{drift, diffusion, previous, checked_exp(log_discount)};
        previous = t;
    }
}

class Planner {
public:
    Planner(const Model& m, const kgpu_note* notes, int count, const kgpu_note_observation* obs, const double* mon)
        : m_(m), notes_(notes), count_(count), obs_(obs), mon_(mon) {}

    Note note(int i) const {
        Note v;
        v.n = &notes_[i];
        v.obs = obs_ + notes_[i].observation_offset;
        v.obs_count = notes_[i].observation_count;
        if (notes_[i].flags & KGPU_NOTE_MONITORING) {
            v.mon = mon_ + notes_[i].monitoring_offset;
            v.mon_count = notes_[i].monitoring_count;
        }
        return v;
    }

    // shared_lane (DailyGrids::prepare, portfolio.rs:74-185): the note's plan on its
    // daily grid, or false for a scalar quote.
    bool lane(int i, Lane& out) {
        const Note note = this->note(i);
        const kgpu_note& n = *note.n;
        const double spot = m_.spot;
        // _daily: daily monitoring that still matters, not knocked in at valuation
        if (!(note.daily_knock_in() && note.knock_in_affects_payoff())) return false;
        try {
            if (!prior_ok(note)) return false;
            const Initial state = initial_state(note, spot);
            if (state.knocked_in) return false;
            if (state.settles || fixed_value(note, spot, m_.rate, state.knocked_in)) return false;
            // prepare_sample_on_grid without the bridge plan
            const Grid& g = grid(note);
            out = Lane{};
            out.note = i;
            out.grid = &g;
            out.steps = int(g.times.size());
            kgpu_contract& c = out.contract;
            c.payoff = KGPU_PAYOFF_AUTOCALLABLE;
            c.sign = 1.0;
            c.spot = spot;
            int flag = KGPU_C_HAS_KNOCK_IN;
            const bool expiry_knock_in = !note.monitored() || (note.mon_count > 0 && note.mon[note.mon_count - 1] == n.expiry);
            if (expiry_knock_in) flag |= KGPU_C_EXPIRY_KNOCK_IN;
            if (!note.fixed()) flag |= KGPU_C_DOWNSIDE;
            c.flags = flag;
            c.step_count = out.steps;
            c.knock_in = log_ratio(n.knock_in_level, spot);
            c.initial_cash = state.coupon;
            c.terminal_base = n.principal + note.rebate_payment(n.expiry);
            c.terminal_plain = note.terminal(0.0, false);
            c.terminal_fixed = note.fixed() ? note.terminal(0.0, true) : 0.0;
            c.downside_lower = n.lower_strike;
            c.downside_upper = n.upper_strike;
            c.downside_initial = n.initial_spot;
            c.final_discount = checked_exp(-m_.rate * g.times.back());
            int events = 0;
            out.events.reserve(size_t(note.obs_count));
            for (int k = 0; k < note.obs_count; ++k) {
                const kgpu_note_observation& o = note.obs[k];
                if (!(o.time > 0.0)) continue;
                const int step = int(std::lower_bound(g.times.begin(), g.times.end(), o.time) - g.times.begin());
                out.events.push_back(cash_event(note, o, spot, m_.rate, step));
                ++events;
            }
            c.event_count = events;
        } catch (const Defer&) {
            return false;
        }
        // the monitoring dates after valuation; every cash event on one of them or expiry
        bool any_future = false;
        double last_future = 0.0;
        for (int k = 0; k < note.mon_count; ++k)
            if (note.mon[k] > 0.0) {
                any_future = true;
                last_future = note.mon[k];
            }
        bool on_grid = any_future;
        for (int k = 0; k < note.obs_count && on_grid; ++k) {
            const double t = note.obs[k].time;
            if (t > 0.0 && !(t == n.expiry || note.monitors(t))) on_grid = false;
        }
        if (!on_grid) {
            bool observes = false;
            for (uint8_t f : out.grid->knock_in) observes = observes || (f & KGPU_STEP_KNOCK_IN);
            if (!observes) return false;
            out.sparse = false;
            out.maturity_on_grid = false;
            return true;
        }
        out.sparse = true;
        out.maturity_on_grid = last_future == n.expiry;
        return true;
    }

private:
    // _event_grid: the note's merged grid, shared by notes with the same event dates,
    // monitoring range and expiry.
    const Grid& grid(const Note& note) {
        std::vector<double>& key = key_;
        key.clear();
        key.push_back(note.n->expiry);
        key.push_back(double(note.n->monitoring_offset));
        key.push_back(double(note.mon_count));
        for (int k = 0; k < note.obs_count; ++k)
            if (note.obs[k].time > 0.0) key.push_back(note.obs[k].time);
        std::string& bytes = key_bytes_;
        bytes.assign(reinterpret_cast<const char*>(key.data()), key.size() * sizeof(double));
        auto hit = grids_.find(bytes);
        if (hit != grids_.end()) return hit->second;
        Grid g;
        for (int k = 0; k < note.obs_count; ++k)
            if (note.obs[k].time > 0.0) g.times.push_back(note.obs[k].time);
        for (int k = 0; k < note.mon_count; ++k)
            if (note.mon[k] > 0.0) g.times.push_back(note.mon[k]);
        if (note.n->expiry > 0.0) g.times.push_back(note.n->expiry);
        std::sort(g.times.begin(), g.times.end());
        g.times.erase(std::unique(g.times.begin(), g.times.end()), g.times.end());
        grid_steps(m_, g);
        g.knock_in.assign(g.times.size(), 0);
        for (size_t i = 0; i < g.times.size(); ++i)
            if (note.monitors(g.times[i])) g.knock_in[i] = KGPU_STEP_KNOCK_IN;
        return grids_.emplace(bytes, std::move(g)).first->second;
    }

    Model m_;
    const kgpu_note* notes_;
    int count_;
    const kgpu_note_observation* obs_;
    const double* mon_;
    std::unordered_map<std::string, Grid> grids_;
    std::vector<double> key_;
    std::string key_bytes_;
};

// same_daily_grid (portfolio.rs:872-901): equal transitions and monitoring flags on the
// common dates; grids of different lengths must both end on their maturity.
bool same_daily_grid(const Lane& a, const Lane& b) {
    if (a.steps != b.steps && !(a.sparse && a.maturity_on_grid && b.sparse && b.maturity_on_grid)) return false;
    if (a.grid == b.grid) return true;  // one grid object: equal records and flags
    const int n = std::min(a.steps, b.steps);
    for (int i = 0; i < n; ++i) {
        const kgpu_step& x = a.grid->steps[i];
        const kgpu_step& y = b.grid->steps[i];
        if (std::memcmp(&x.drift, &y.drift, sizeof(double)) || std::memcmp(&x.diffusion, &y.diffusion, sizeof(double)) ||
            std::memcmp(&x.discount, &y.discount, sizeof(double)))
            return false;
        if (a.grid->knock_in[i] != b.grid->knock_in[i]) return false;
    }
    return true;
}

// The grouping key of a grid that is not an aligned daily grid: its transitions and
// monitoring flags (portfolio.rs:124-131, 438-458).
uint64_t grid_hash(const Lane& lane) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        for (size_t k = 0; k < n; ++k) h = (h ^ b[k]) * 1099511628211ull;
    };
    mix(&lane.steps, sizeof(lane.steps));
    for (int i = 0; i < lane.steps; ++i) {
        const kgpu_step& s = lane.grid->steps[i];
        mix(&s.drift, sizeof(double));
        mix(&s.diffusion, sizeof(double));
        mix(&s.discount, sizeof(double));
        mix(&lane.grid->knock_in[i], 1);
    }
    return h;
}

// Terms equality for coupon families: every term but the portfolio coupon, with whether
// knock-in changes the payoff (portfolio_family_key and shares_portfolio_terms,
// instruments/autocallable.rs:1188-1300).  Doubles compare by value.
struct FamilyKey {
    const Note* note;
    bool phoenix;
};

uint64_t hash_double(uint64_t h, double x) {
    if (x == 0.0) x = 0.0;  // 0.0 and -0.0 are one key
    uint64_t bits;
    std::memcpy(&bits, &x, sizeof(bits));
    h ^= bits + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    return h;
}

uint64_t family_hash(const Note& a, bool phoenix) {
    const kgpu_note& n = *a.n;
    uint64_t h = phoenix ? 1 : 2;
    h = hash_double(h, n.initial_spot);
    h = hash_double(h, n.expiry);
    h = hash_double(h, a.has_ki() ? n.knock_in_level : 0.0);
    h = hash_double(h, n.upper_strike);
    h = hash_double(h, n.lower_strike);
    if (phoenix) h = hash_double(h, n.maturity_coupon_rate);
    else h = hash_double(h, n.period_coupon);
    h = hash_double(h, n.principal);
    h = hash_double(h, double(n.flags) + 8.0 * n.barrier_state + 64.0 * a.obs_count + 1e6 * a.mon_count);
    for (int k = 0; k < a.obs_count; ++k) {
        h = hash_double(h, a.obs[k].time);
        h = hash_double(h, a.obs[k].coupon_rate);
    }
    return h;
}

bool same_option(bool has_a, double a, bool has_b, double b) { return has_a == has_b && (!has_a || a == b); }

bool same_family(const Note& a, bool pa, const Note& b, bool pb) {
    if (pa != pb) return false;
    const kgpu_note& x = *a.n;
    const kgpu_note& y = *b.n;
    if (!(x.initial_spot == y.initial_spot && x.expiry == y.expiry && x.upper_strike == y.upper_strike &&
          x.lower_strike == y.lower_strike && x.principal == y.principal && x.rebate_rate == y.rebate_rate &&
          x.annual_rebate_rate == y.annual_rebate_rate && x.effective_time == y.effective_time &&
          x.barrier_state == y.barrier_state))
        return false;
    if (pa ? x.maturity_coupon_rate != y.maturity_coupon_rate : x.period_coupon != y.period_coupon) return false;
    if (!same_option(a.has_ki(), x.knock_in_level, b.has_ki(), y.knock_in_level)) return false;
    if (!same_option(a.fixed(), x.fixed_knock_in_coupon, b.fixed(), y.fixed_knock_in_coupon)) return false;
    if (a.monitored() != b.monitored() || a.mon_count != b.mon_count) return false;
    if (a.mon != b.mon)
        for (int k = 0; k < a.mon_count; ++k)
            if (a.mon[k] != b.mon[k]) return false;
    if (a.obs_count != b.obs_count) return false;
    for (int k = 0; k < a.obs_count; ++k) {
        const kgpu_note_observation& o = a.obs[k];
        const kgpu_note_observation& p = b.obs[k];
        if (o.time != p.time || o.coupon_rate != p.coupon_rate) return false;
        if (!same_option(Note::has_ko(o), o.knock_out_level, Note::has_ko(p), p.knock_out_level)) return false;
        if (!same_option(Note::has_cb(o), o.coupon_barrier_level, Note::has_cb(p), p.coupon_barrier_level)) return false;
    }
    return a.knock_in_affects_payoff() == b.knock_in_affects_payoff();
}

bool fp32_ok(double v) {
    const double a = std::fabs(v);
    return a == 0.0 || !std::isfinite(a) || (a >= 0x1p-100 && a <= 0x1p120);
}

struct GroupFailure {
    kgpu_status status;
    const char* message;
};

// SharedEvents::new (portfolio.rs:903-1047) and the lanes' contracts, packed.
void plan_group(const std::vector<const Lane*>& lanes, double spot, kgpu_shared_plan::Group& out,
                std::vector<uint8_t>& fp32) {
    const Lane* base = lanes[0];
    for (const Lane* l : lanes)
        if (l->steps >= base->steps) base = l;  // the last of the longest grids
    const int n = base->steps;
    const std::vector<kgpu_step>& steps = base->grid->steps;
    std::vector<char> action(n, 0);
    for (const Lane* l : lanes) {
        for (const kgpu_event& e : l->events) action[e.step] = 1;
        action[l->steps - 1] = 1;
    }
    double excursion = 0.0;
    for (int i = 0; i < n; ++i) excursion += std::fabs(steps[i].drift) + 20.0 * steps[i].diffusion;
    double low, high;
    safe_log_returns(spot, &low, &high);
    const bool bridge = low <= excursion && excursion <= high && low <= -excursion && -excursion <= high;
    std::vector<kgpu_bridge_daily> daily(n, kgpu_bridge_daily{0.0, 0.0});
    std::vector<kgpu_bridge_interval> intervals;
    std::vector<kgpu_bridge_daily> weights;
    int first = 0;
    for (int step = 0; step < n; ++step) {
        if (!action[step] && step + 1 < n) continue;
        if (bridge && step - first >= 8) {
            double total = steps[step].drift;
            double variance = steps[step].diffusion * steps[step].diffusion;
            weights.assign(size_t(step - first), kgpu_bridge_daily{0.0, 0.0});
            for (int i = step - 1; i >= first; --i) {
                const double w = steps[i].diffusion;
                const double next = std::fma(w, w, variance);
                // 0 / 0 (a vanishing width) is NaN, which refuses the bridge below
                weights[i - first] = kgpu_bridge_daily{next == 0.0 ? kNan : (w * w) / next,
                                                       next == 0.0 ? kNan : w * std::sqrt(variance / next)};
                total += steps[i].drift;
                variance = next;
            }
            const double diffusion = std::sqrt(variance);
            bool positive = true;
            for (const kgpu_bridge_daily& d : weights) positive = positive && d.weight > 0.0 && d.width > 0.0;
            if (is_normal(diffusion) && std::isfinite(total) && positive) {
                for (int i = first; i < step; ++i) {
                    if (!(base->grid->knock_in[i] & KGPU_STEP_KNOCK_IN))
                        throw GroupFailure{KGPU_COMPUTATION_FAILURE, "a bridged day does not monitor knock-in"};
                    daily[i] = weights[i - first];
                }
                intervals.push_back(kgpu_bridge_interval{step, 0, total, diffusion});
                first = step + 1;
                continue;
            }
        }
        for (int i = first; i <= step; ++i) intervals.push_back(kgpu_bridge_interval{i, 0, steps[i].drift, steps[i].diffusion});
        first = step + 1;
    }
    // Interval checks of the FP32 rule, per prefix length.
    std::vector<uint8_t> interval_ok(intervals.size() + 1, 1);
    for (size_t q = 0; q < intervals.size(); ++q)
        interval_ok[q + 1] = interval_ok[q] && fp32_ok(intervals[q].drift) && fp32_ok(intervals[q].diffusion);
    // lane_plans: one bridged contract per lane; lanes of one maturity and event steps
    // share one segment of steps, flags and bridge weights.
    // Segments by (maturity, event steps); a lane joins one whose step records equal its
    // own (the records' times included).
    struct Segment {
        int64_t offset;
        bool fp32;
        const Grid* grid;  // the grid whose records the segment copied
    };
    std::map<std::vector<int>, std::vector<Segment>> segments;
    std::vector<int> key;
    std::vector<const Grid*> prefixes{base->grid};  // grids checked against the base
    out.intervals = intervals;
    for (const Lane* l : lanes) {
        const int m = l->steps - 1;
        const kgpu_step* own_steps = l->grid->steps.data();
        if (std::find(prefixes.begin(), prefixes.end(), l->grid) == prefixes.end()) {
            for (int i = 0; i <= m; ++i)
                if (l->grid->knock_in[i] != base->grid->knock_in[i] ||
                    std::memcmp(&own_steps[i].drift, &steps[i].drift, sizeof(double)) != 0 ||
                    std::memcmp(&own_steps[i].diffusion, &steps[i].diffusion, sizeof(double)) != 0 ||
                    std::memcmp(&own_steps[i].discount, &steps[i].discount, sizeof(double)) != 0)
                    throw GroupFailure{KGPU_INVALID_INPUT, "the lanes do not share one daily grid"};
            prefixes.push_back(l->grid);
        }
        int own = 0;
        while (own < int(intervals.size()) && intervals[own].end <= m) ++own;
        if (own == 0 || intervals[own - 1].end != m)
            throw GroupFailure{KGPU_COMPUTATION_FAILURE, "a lane's maturity does not end an interval"};
        key.assign(1, m);
        for (const kgpu_event& e : l->events) key.push_back(e.step);
        std::vector<Segment>& candidates = segments[key];
        const Segment* seg = nullptr;
        for (const Segment& c : candidates)
            if (c.grid == l->grid ||
                std::memcmp(out.steps.data() + c.offset, own_steps, sizeof(kgpu_step) * size_t(m + 1)) == 0) {
                seg = &c;
                break;
            }
        if (!seg) {
            const int64_t offset = int64_t(out.steps.size());
            bool ok = true;
            for (int i = 0; i <= m; ++i) {
                out.steps.push_back(own_steps[i]);
                out.flags.push_back(l->grid->knock_in[i]);
                out.daily.push_back(daily[i]);
                ok = ok && fp32_ok(own_steps[i].drift) && fp32_ok(own_steps[i].diffusion) &&
                     fp32_ok(own_steps[i].discount) && fp32_ok(daily[i].weight) && fp32_ok(daily[i].width);
            }
            for (const kgpu_event& e : l->events) out.flags[size_t(offset) + e.step] |= KGPU_STEP_EVENT;
            candidates.push_back(Segment{offset, ok, l->grid});
            seg = &candidates.back();
        }
        kgpu_contract c = l->contract;
        c.step_count = m + 1;
        c.step_offset = seg->offset;
        c.event_offset = int32_t(out.events.size());
        c.event_count = int32_t(l->events.size());
        c.flags = (c.flags & ~KGPU_C_BRIDGE) | KGPU_C_BRIDGE;
        c.bridge_offset = 0;
        c.bridge_count = own;
        c.final_discount = steps[m].discount;
        c.dimensions = n;
        bool ok = seg->fp32 && interval_ok[own];
        for (const double* v = &c.strike; v <= &c.greek_log_weight; ++v) ok = ok && fp32_ok(*v);
        for (const kgpu_event& e : l->events) {
            ok = ok && fp32_ok(e.knock_out) && fp32_ok(e.coupon_barrier);
            for (double p : e.payment) ok = ok && fp32_ok(p);
            out.events.push_back(e);
        }
        fp32.push_back(ok ? 1 : 0);
        out.contracts.push_back(c);
    }
}

kgpu_status fail(kgpu_status status, const char* message) {
    kgpu::set_thread_error(message);
    return status;
}

}  // namespace

extern "C" {

kgpu_status kgpu_shared_plan_create(const kgpu_model* model, const kgpu_note* notes, int32_t note_count,
                                    const kgpu_note_observation* observations, int32_t observation_total,
                                    const double* monitoring, int32_t monitoring_total, const uint8_t* simulate,
                                    kgpu_shared_plan** out) {
    if (!out) return fail(KGPU_INVALID_INPUT, "out must not be null");
    *out = nullptr;
    if (!model || note_count < 0 || (note_count > 0 && !notes) || observation_total < 0 || monitoring_total < 0 ||
        (observation_total > 0 && !observations) || (monitoring_total > 0 && !monitoring))
        return fail(KGPU_INVALID_INPUT, "null or negative arguments");
    if (note_count > (1 << 20)) return fail(KGPU_INVALID_INPUT, "contract batch exceeds 1,048,576 instruments");
    if (!(model->spot > 0.0 && std::isfinite(model->spot))) return fail(KGPU_INVALID_INPUT, "spot must be positive and finite");
    for (int i = 0; i < note_count; ++i) {
        const kgpu_note& n = notes[i];
        if (n.observation_offset < 0 || n.observation_count < 0 ||
            int64_t(n.observation_offset) + n.observation_count > observation_total)
            return fail(KGPU_INVALID_INPUT, "a note's observations lie outside the observation table");
        if ((n.flags & KGPU_NOTE_MONITORING) &&
            (n.monitoring_offset < 0 || n.monitoring_count < 0 ||
             int64_t(n.monitoring_offset) + n.monitoring_count > monitoring_total))
            return fail(KGPU_INVALID_INPUT, "a note's monitoring times lie outside the monitoring table");
        if (n.barrier_state < KGPU_STATE_UNKNOWN || n.barrier_state > KGPU_STATE_KNOCKED_OUT)
            return fail(KGPU_INVALID_INPUT, "unknown barrier state");
    }
    // Monitoring times strictly increasing (validate_life and the schedule checks of the
    // instrument), checked once per distinct range.
    {
        std::unordered_map<int64_t, int32_t> checked;
        for (int i = 0; i < note_count; ++i) {
            const kgpu_note& n = notes[i];
            if (!(n.flags & KGPU_NOTE_MONITORING) || n.monitoring_count < 2) continue;
            auto hit = checked.find(n.monitoring_offset);
            if (hit != checked.end() && hit->second >= n.monitoring_count) continue;
            for (int k = 1; k < n.monitoring_count; ++k)
                if (!(monitoring[n.monitoring_offset + k - 1] < monitoring[n.monitoring_offset + k]))
                    return fail(KGPU_INVALID_INPUT, "knock-in monitoring times must be strictly increasing");
            checked[n.monitoring_offset] = n.monitoring_count;
        }
    }
    kgpu_shared_plan* plan = new (std::nothrow) kgpu_shared_plan;
    if (!plan) return fail(KGPU_DEVICE_ERROR, "out of host memory");
    try {
        const int n = note_count;
        plan->note_count = n;
        plan->note_group.assign(size_t(n), -1);
        plan->coupon.assign(size_t(n), 0.0);
        plan->simulated.assign(size_t(n), 0);
        plan->group_first_lane.push_back(0);
        if (model->kind == KGPU_MODEL_BSM) {
            const Model m{model->spot, model->rate, model->dividend, model->volatility};
            Planner planner(m, notes, n, observations, monitoring);
            // Lanes and their groups, in book order (plan_book, portfolio.rs:187-318).
            std::vector<Lane> lanes;
            lanes.reserve(size_t(n));
            std::vector<std::vector<int>> groups;        // lane indices
            std::vector<int> daily_groups;               // groups of aligned daily grids
            std::unordered_map<uint64_t, std::vector<int>> grid_groups;
            // same_daily_grid depends only on the two lanes' grid objects and alignment
            std::map<std::tuple<const Grid*, const Grid*, bool, bool>, bool> compared;
            auto same_grid = [&](const Lane& a, const Lane& b) {
                if (a.grid == b.grid) return same_daily_grid(a, b);
                const auto key = std::make_tuple(a.grid, b.grid, a.sparse && a.maturity_on_grid,
                                                 b.sparse && b.maturity_on_grid);
                auto hit = compared.find(key);
                if (hit != compared.end()) return hit->second;
                const bool same = same_daily_grid(a, b);
                compared.emplace(key, same);
                return same;
            };
            Lane lane;
            for (int i = 0; i < n; ++i) {
                if (!planner.lane(i, lane)) continue;
                lanes.push_back(std::move(lane));
                const int li = int(lanes.size()) - 1;
                const Lane& l = lanes.back();
                std::vector<int>& candidates =
                    l.sparse && l.maturity_on_grid ? daily_groups : grid_groups[grid_hash(l)];
                bool placed = false;
                for (int g : candidates)
                    if (same_grid(lanes[size_t(groups[size_t(g)][0])], l)) {
                        groups[size_t(g)].push_back(li);
                        placed = true;
                        break;
                    }
                if (!placed) {
                    candidates.push_back(int(groups.size()));
                    groups.push_back({li});
                }
            }
            std::vector<Note> views(static_cast<size_t>(n));
            for (int i = 0; i < n; ++i) views[size_t(i)] = planner.note(i);
            for (const std::vector<int>& members : groups) {
                if (members.size() == 1) continue;  // a singleton takes the scalar estimator
                const int g = int(plan->groups.size());
                std::vector<uint8_t> sim(members.size(), 1);
                if (members.size() >= 3) {
                    // coupon families (price_coupon_families, portfolio.rs:570-667)
                    std::vector<std::vector<int>> families;  // group positions
                    std::unordered_map<uint64_t, std::vector<int>> by_hash;
                    std::vector<uint8_t> phoenix(members.size());
                    std::vector<double> coupon(members.size());
                    for (size_t p = 0; p < members.size(); ++p) {
                        const Note& v = views[size_t(lanes[size_t(members[p])].note)];
                        phoenix[p] = v.phoenix();
                        coupon[p] = phoenix[p] ? v.n->period_coupon : v.n->maturity_coupon_rate;
                        std::vector<int>& bucket = by_hash[family_hash(v, phoenix[p])];
                        bool found = false;
                        for (int f : bucket) {
                            const int q = families[size_t(f)][0];
                            if (same_family(views[size_t(lanes[size_t(members[size_t(q)])].note)], phoenix[size_t(q)], v,
                                            phoenix[p])) {
                                families[size_t(f)].push_back(int(p));
                                found = true;
                                break;
                            }
                        }
                        if (!found) {
                            bucket.push_back(int(families.size()));
                            families.push_back({int(p)});
                        }
                    }
                    for (const std::vector<int>& family : families) {
                        if (family.size() < 3) continue;
                        int lo = family[0], hi = family[1];
                        if (coupon[size_t(lo)] > coupon[size_t(hi)]) std::swap(lo, hi);
                        for (size_t k = 2; k < family.size(); ++k) {
                            const int p = family[k];
                            if (coupon[size_t(p)] < coupon[size_t(lo)]) lo = p;
                            if (coupon[size_t(p)] > coupon[size_t(hi)]) hi = p;
                        }
                        const double width = coupon[size_t(hi)] - coupon[size_t(lo)];
                        if (!std::isfinite(width)) continue;
                        kgpu_shared_plan::Strip strip;
                        strip.low = lanes[size_t(members[size_t(lo)])].note;
                        strip.high = lanes[size_t(members[size_t(hi)])].note;
                        strip.width = width;
                        for (int p : family) {
                            strip.members.push_back(lanes[size_t(members[size_t(p)])].note);
                            sim[size_t(p)] = (p == lo || p == hi) ? 1 : 0;
                        }
                        plan->strips.push_back(std::move(strip));
                    }
                    for (size_t p = 0; p < members.size(); ++p)
                        plan->coupon[size_t(lanes[size_t(members[p])].note)] = coupon[p];
                }
                std::vector<const Lane*> simulated;
                for (size_t p = 0; p < members.size(); ++p) {
                    const int note = lanes[size_t(members[p])].note;
                    plan->note_group[size_t(note)] = g;
                    if (simulate && simulate[note]) sim[p] = 1;
                    plan->simulated[size_t(note)] = sim[p];
                    if (sim[p]) simulated.push_back(&lanes[size_t(members[p])]);
                }
                plan->groups.emplace_back();
                kgpu_status status = KGPU_OK;
                const char* message = "";
                const size_t fp32_before = plan->lane_fp32.size();
                try {
                    plan_group(simulated, m.spot, plan->groups.back(), plan->lane_fp32);
                } catch (const GroupFailure& f) {
                    status = f.status;
                    message = f.message;
                    plan->groups.back() = kgpu_shared_plan::Group{};
                    plan->lane_fp32.resize(fp32_before);
                }
                if (status == KGPU_OK)
                    for (const Lane* l : simulated) plan->lane_note.push_back(l->note);
                plan->group_status.push_back(status);
                plan->message_text.push_back(message);
                plan->group_first_lane.push_back(int32_t(plan->lane_note.size()));
            }
        }
        for (kgpu_shared_plan::Group& g : plan->groups) {
            kgpu_book b{};
            b.contract_count = int32_t(g.contracts.size());
            b.contracts = g.contracts.data();
            b.step_total = int64_t(g.steps.size());
            b.steps = g.steps.data();
            b.step_flags = g.flags.data();
            b.bridge_daily = g.daily.empty() ? nullptr : g.daily.data();
            b.event_total = int32_t(g.events.size());
            b.interval_total = int32_t(g.intervals.size());
            b.events = g.events.empty() ? nullptr : g.events.data();
            b.intervals = g.intervals.empty() ? nullptr : g.intervals.data();
            plan->group_books.push_back(b);
        }
        for (const std::string& s : plan->message_text) plan->group_message.push_back(s.c_str());
    } catch (const std::bad_alloc&) {
        delete plan;
        return fail(KGPU_DEVICE_ERROR, "out of host memory");
    }
    *out = plan;
    return KGPU_OK;
}

kgpu_status kgpu_shared_plan_get(const kgpu_shared_plan* plan, kgpu_shared_plan_view* out) {
    if (!plan || !out) return fail(KGPU_INVALID_INPUT, "plan and out must not be null");
    kgpu_shared_plan_view v{};
    v.note_count = plan->note_count;
    v.group_count = int32_t(plan->groups.size());
    v.lane_count = int32_t(plan->lane_note.size());
    v.note_group = plan->note_group.data();
    v.group_first_lane = plan->group_first_lane.data();
    v.lane_note = plan->lane_note.data();
    v.lane_fp32 = plan->lane_fp32.data();
    v.group_books = plan->group_books.data();
    v.group_status = plan->group_status.data();
    v.group_message = plan->group_message.data();
    *out = v;
    return KGPU_OK;
}

kgpu_status kgpu_shared_plan_interpolate(const kgpu_shared_plan* plan, double* note_prices, uint8_t* retry) {
    if (!plan || (plan->note_count > 0 && (!note_prices || !retry)))
        return fail(KGPU_INVALID_INPUT, "plan, note_prices and retry must not be null");
    if (plan->note_count == 0) return KGPU_OK;
    std::memset(retry, 0, size_t(plan->note_count));
    for (const kgpu_shared_plan::Strip& strip : plan->strips) {
        const double lower = note_prices[strip.low];
        const double upper = note_prices[strip.high];
        const double c_low = plan->coupon[size_t(strip.low)];
        for (int32_t i : strip.members) {
            if (plan->simulated[size_t(i)]) continue;
            const double fraction = strip.width > 0.0 ? (plan->coupon[size_t(i)] - c_low) / strip.width : 0.0;
            const double a = lower * (1.0 - fraction), b = upper * fraction;
            const double price = a + b;
            const double magnitude = std::fabs(a) + std::fabs(b);
            if (!std::isfinite(price) || std::fabs(price) < 1e-12 * magnitude)
                retry[i] = 1;
            else
                note_prices[i] = price;
        }
    }
    return KGPU_OK;
}

void kgpu_shared_plan_destroy(kgpu_shared_plan* plan) { delete plan; }

}  // extern "C"
