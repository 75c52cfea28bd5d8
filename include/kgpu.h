/*
 * kiyosi-gb300 C ABI: GB300 (sm_103a) Monte Carlo and least-squares Monte Carlo
 * pricing engines for kiyosi, behind plain pointers, sizes and status codes.
 *
 * The host side that replaces the reference's Rust engines builds a *plan* for each
 * contract -- the same per-step transitions, cash events and thresholds that the
 * reference's engines build before their sampling loops -- and hands the plans to
 * this library.  The library owns all device memory; every output buffer is
 * caller-owned host memory.  No C++ exception and no torch type crosses this ABI.
 *
 * Reference interfaces replaced (paths inside the kiyosi crate):
 *   PricingEngine::{price, price_with_seed, price_with_statistics}
 *       crates/kiyosi/src/risk/analytics.rs:771,782,796
 *   MonteCarloVanillaEngine (European)       engines/monte_carlo.rs:1093-1141,1254-1330
 *   MonteCarloAutocallableEngine::{price, price_many}
 *                                             engines/monte_carlo/autocallable.rs:119-152,293-430
 *   MonteCarloAccumulatorEngine               engines/monte_carlo/accumulator.rs:91-218
 *   MonteCarloDigitalEngine                   engines/monte_carlo/digital.rs:55-130
 *   MonteCarloVanillaEngine (American, LSMC)  engines/monte_carlo/american.rs:955-1455
 *   MonteCarloEstimate / status               engines/monte_carlo.rs:858-1001
 *   Error variants                            crates/kiyosi/src/error.rs:19-48
 */
#ifndef KIYOSI_GB300_KGPU_H
#define KIYOSI_GB300_KGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KGPU_ABI_VERSION 1

/* Status codes map one-to-one onto kiyosi's Error variants (error.rs:19-48), plus a
 * device error.  KGPU_INTERRUPTED is Error::Io(Interrupted) from cancellation. */
typedef enum kgpu_status {
    KGPU_OK = 0,
    KGPU_INVALID_INPUT = 1,
    KGPU_MISSING_HISTORY = 2,
    KGPU_UNSUPPORTED_OPERATION = 3,
    KGPU_GREEK_UNAVAILABLE = 4,
    KGPU_COMPUTATION_FAILURE = 5,
    KGPU_ROOT_NOT_BRACKETED = 6,
    KGPU_INTERRUPTED = 7,
    KGPU_DEVICE_ERROR = 8
} kgpu_status;

/* MonteCarloSampling (monte_carlo.rs:71-80). */
enum { KGPU_SAMPLING_PSEUDO_RANDOM = 0, KGPU_SAMPLING_SOBOL = 1 };

/* Arithmetic of the path kernels.  FP64 follows the reference's arithmetic step for step.
 * FP32 steps paths in single precision; each path's payoff is widened to FP64 before any
 * addition, and every sum (per block, across blocks) is an FP64 sum in a fixed order.
 * An FP64 sum of FP32 payoffs carries less rounding than a compensated FP32 running sum
 * would, so no per-thread FP32 accumulator exists. */
enum { KGPU_PRECISION_FP64 = 0, KGPU_PRECISION_FP32 = 1 };

/* Launch schedule.  PLAIN: one contract per launch, one thread per sample, the
 * reference's 256-sample blocks as CUDA blocks, sequential scaled-Welford moments per
 * block merged in block order.  PERSISTENT: the whole book at once.  A book whose every
 * contract is a Brownian-bridged autocallable (KGPU_C_BRIDGE, BSM) runs phase-major in
 * FP32, as one cooperative launch: each grid step advances every path still monitoring
 * knock-in by one bridge interval, the lanes of a warp on the same grid positions, and
 * the survivors go to the next step's list; once few paths remain, CTAs complete them,
 * then the knocked-in paths (interval ends only).  In FP32 under PCG32, a book of BSM
 * vanilla paths runs eight lanes per path (the path's steps in segments, the segment sums
 * added in a fixed order: prices within 1e-5 relative), and any other book of Asians and
 * vanilla paths one thread per path.  Other books (and FP64) run the lane-refill kernel:
 * warps pull (contract, tile) work items from a device queue and refill finished lanes
 * with the next path of the tile.
 * LANE_REFILL: the lane-refill kernel for every book.  The persistent kernels store each
 * path's payoff and sum the payoffs in a fixed order, so the phase-major and lane-refill
 * estimates are identical for a book both can run. */
/* KGPU_SCHEDULE_SHARED_GRID: the book's contracts are the lanes of one shared daily grid
 * (bridged autocallables whose steps, bridge intervals and bridge weights are prefixes of
 * the longest lane's, with equal sampling dimensions and path counts).  One thread per
 * path walks the longest lane's plan once and settles every lane on it; the estimates
 * equal those of the plain schedule up to the order of the sums.  Pseudo-random or
 * Sobol, with or without antithetic pairs; host-resident books only. */
enum {
    KGPU_SCHEDULE_PLAIN = 0,
    KGPU_SCHEDULE_PERSISTENT = 1,
    KGPU_SCHEDULE_SHARED_GRID = 2,
    KGPU_SCHEDULE_LANE_REFILL = 3
};

/* MonteCarloSettings (monte_carlo.rs:86-105) plus the GPU controls. */
typedef struct kgpu_settings {
    int32_t path_count;   /* default path count; kgpu_contract.path_count > 0 overrides */
    int32_t sampling;     /* KGPU_SAMPLING_* */
    int32_t antithetic;   /* pairs Z and -Z */
    int32_t precision;    /* KGPU_PRECISION_* */
    int32_t schedule;     /* KGPU_SCHEDULE_* */
    int32_t tile_paths;   /* persistent schedule: paths per work item (0 = tuned default;
                             Sobol tiles must divide 256) */
    int32_t ctas_per_sm;  /* persistent schedule: resident CTAs per SM (0 = occupancy limit) */
    int32_t refill;       /* persistent schedule: path units between lane refills (0 = 16) */
    uint64_t seed;        /* resolved seed (the host resolves entropy seeds first) */
} kgpu_settings;

/* Models.  Rates are flat, as every reference MC engine requires (engines.rs:133-136). */
enum { KGPU_MODEL_BSM = 0, KGPU_MODEL_HESTON = 1, KGPU_MODEL_LOCAL_VOL = 2 };

typedef struct kgpu_model {
    int32_t kind;           /* KGPU_MODEL_* */
    int32_t lv_time_count;  /* local volatility: >= 2 time nodes */
    int32_t lv_spot_count;  /* local volatility: >= 2 spot nodes */
    int32_t reserved;
    double spot;            /* spot at valuation */
    double rate;            /* flat risk-free rate */
    double dividend;        /* flat dividend yield */
    double volatility;      /* BSM sigma */
    double v0, kappa, theta, xi, rho;  /* Heston (market/heston.rs:58-227) */
    /* Local volatility surface (market/local_volatility.rs:322-359): bilinear in (years
     * since lv_times[0], absolute spot) with both axes clamped; values[time][spot]. */
    const double* lv_times;
    const double* lv_spots;
    const double* lv_values;
} kgpu_model;

/* Payoff families. */
enum {
    KGPU_PAYOFF_EUROPEAN = 0,     /* exact terminal sampling, one dimension (monte_carlo.rs:1165-1252) */
    KGPU_PAYOFF_VANILLA_PATH = 1, /* vanilla payoff of the spot after stepping every grid step */
    KGPU_PAYOFF_ASIAN = 2,        /* arithmetic average of the spots at FIXING steps */
    KGPU_PAYOFF_AUTOCALLABLE = 3, /* snowball / phoenix / binary / ternary (autocallable.rs:823-862) */
    KGPU_PAYOFF_ACCUMULATOR = 4,  /* accumulator.rs:160-216 */
    KGPU_PAYOFF_DIGITAL = 5,      /* terminal digital, one dimension (digital.rs:111-130) */
    KGPU_PAYOFF_BARRIER = 6,      /* continuously monitored single barrier: one terminal draw
                                     and Brownian-bridge survival (barrier.rs:231-452) */
    KGPU_PAYOFF_BARRIER_DISCRETE = 7, /* single barrier observed on dates (barrier.rs:231-452):
                                     one step per date; one kgpu_event per step holds the
                                     date's record (see kgpu_contract) */
    KGPU_PAYOFF_AVERAGE_ARITHMETIC = 8, /* continuous arithmetic average (asian.rs:374-713,
                                     1016-1257): trapezoid over n intervals, the first one
                                     integrated analytically, n - 1 (+ lead) normals */
    KGPU_PAYOFF_AVERAGE_GEOMETRIC = 9, /* continuous geometric average or single fixing:
                                     one exact normal (asian.rs:740-784) */
    KGPU_PAYOFF_DOUBLE_BARRIER = 10 /* continuously monitored double barrier: one terminal
                                     draw weighted by the killed-density survival series
                                     (barrier.rs:341-390, double_barrier.rs:6-112) */
};

/* One simulated grid step of a contract.  For BSM the transition is the reference's
 * transition() (monte_carlo.rs:2123-2137) computed on the host:
 *   drift = (r - q - sigma^2/2) dt,  diffusion = sigma sqrt(dt).
 * For Heston and local volatility drift = dt and diffusion = sqrt(dt); the kernel
 * forms the state-dependent transition.  `time` is the step's start in years since
 * valuation, `discount` the discount factor exp(-r t_end) at the step's end. */
typedef struct kgpu_step {
    double drift;
    double diffusion;
    double time;
    double discount;
} kgpu_step;

/* Per-step flags (one byte per step, same indexing as kgpu_step). */
enum {
    KGPU_STEP_KNOCK_IN = 1,    /* daily knock-in observation (autocallable) */
    KGPU_STEP_EVENT = 2,       /* cash event (autocallable) or knock-out observation (accumulator) */
    KGPU_STEP_FIXING = 4,      /* Asian fixing */
    KGPU_STEP_ACCUMULATE = 8   /* accumulator purchase date */
};

/* Autocallable cash event (CashEvent, autocallable.rs:524-562).  Thresholds are log
 * returns relative to the valuation spot (numerics.rs:80-92 log_ratio).  payment[k] is
 * the discounted amount for k = coupon_due | (knocked_out << 1), i.e. the reference's
 * discounted_payment() evaluated on the host for the four outcomes. */
typedef struct kgpu_event {
    double knock_out;        /* log KO threshold; ignored unless has_knock_out */
    double coupon_barrier;   /* log coupon threshold */
    double payment[4];
    int32_t has_knock_out;
    int32_t step;            /* grid step index of the event, ascending within a contract */
} kgpu_event;

/* Brownian-bridge plan (BridgePlan, autocallable.rs:451-515).  Intervals end at cash
 * events or expiry; `daily` entries are per grid step (weight, width). */
typedef struct kgpu_bridge_interval {
    int32_t end;        /* grid step index ending the interval */
    int32_t reserved;
    double drift;
    double diffusion;
} kgpu_bridge_interval;

typedef struct kgpu_bridge_daily {
    double weight;      /* fraction of the remaining interval covered by this step */
    double width;       /* sigma sqrt(dt (1 - fraction)) */
} kgpu_bridge_daily;

/* Contract flags. */
enum {
    KGPU_C_HAS_KNOCK_IN = 1,     /* knock_in threshold present */
    KGPU_C_KNOCKED_IN = 2,       /* already knocked in at valuation */
    KGPU_C_EXPIRY_KNOCK_IN = 4,  /* knock-in observed at expiry */
    KGPU_C_DOWNSIDE = 8,         /* knocked-in redemption is the capped downside */
    KGPU_C_BRIDGE = 16,          /* sample with the Brownian bridge plan */
    KGPU_C_ASSET_DIGITAL = 32,   /* digital pays the asset (no payout amount) */
    KGPU_C_BARRIER_UP = 64,      /* barrier above the spot (else below) */
    KGPU_C_BARRIER_IN = 128,     /* knock-in (else knock-out) */
    KGPU_C_REBATE_AT_HIT = 256,  /* discrete knock-out: rebate paid on the hit date */
    KGPU_C_CONDITION_ON_HIT = 512, /* discrete knock-in: after a hit with more than 8 dates left,
                                     the vanilla is priced analytically from the hit */
    KGPU_C_CHECK_STEPS = 1024,    /* discrete barrier whose paths can leave the representable
                                     range: a spot that overflows or underflows fails the
                                     pricing (barrier.rs:280-289) */
    KGPU_C_AVERAGE_LEAD = 2048,   /* arithmetic average starting after valuation: the first
                                     normal draws the lead interval */
    KGPU_C_AVERAGE_CONTROL = 4096, /* arithmetic average with the geometric control variate:
                                     each sample is the residual against the geometric payoff
                                     on the same path; control_mean is added to the mean */
    KGPU_C_DOUBLE = 8192,         /* scheduled double barrier: event payment[3] holds the upper
                                     barrier's touch level (noise >= it touches) */
    KGPU_C_OUTPUT_DELTA = 16384,  /* report each path's likelihood-ratio / pathwise delta sample
                                     instead of its payoff (digital, barrier and average payoffs:
                                     their native delta, digital.rs:116-140, barrier.rs:455-472,
                                     asian.rs:740-784, 1163-1177); the estimate is its mean */
    KGPU_C_OUTPUT_GAMMA = 32768   /* likewise for the gamma sample */
};

/* A contract's plan.  Field groups are used by the payoff families named beside them. */
typedef struct kgpu_contract {
    int32_t payoff;          /* KGPU_PAYOFF_* */
    int32_t flags;           /* KGPU_C_* */
    int32_t path_count;      /* > 0 overrides kgpu_settings.path_count */
    int32_t step_count;      /* simulated steps (sampling dimensions follow from the model) */
    int64_t step_offset;     /* first kgpu_step / flag / bridge daily entry */
    int32_t event_offset;    /* first kgpu_event */
    int32_t event_count;
    int32_t bridge_offset;   /* first kgpu_bridge_interval */
    int32_t bridge_count;
    /* vanilla / Asian / European / digital / accumulator */
    double strike;
    double sign;             /* +1 call, -1 put */
    /* European and digital terminal sampling (EuropeanPayoff::new, monte_carlo.rs:1170-1222) */
    double diffusion;
    double half_variance;
    double moneyness;
    double log_scale;        /* price = mean payoff * exp(log_scale) */
    /* autocallable */
    double knock_in;         /* log KI threshold */
    double initial_cash;     /* coupon fixed at valuation (Initial::coupon) */
    double terminal_base;    /* principal + rebate at expiry */
    double terminal_plain;   /* maturity coupon x accrual when not knocked in */
    double terminal_fixed;   /* fixed coupon x accrual when knocked in (not downside) */
    double downside_lower;   /* settlement strikes and the note's initial spot */
    double downside_upper;
    double downside_initial;
    double final_discount;   /* discount factor at expiry */
    /* accumulator (accumulator.rs:91-218) */
    double knock_out;        /* log KO threshold */
    double quantity;         /* quantity already accrued at valuation */
    double daily_quantity;
    double acceleration;
    double log_strike;       /* log_ratio(strike, spot) */
    /* continuous single barrier (barrier.rs:231-452); strike, sign, diffusion (sigma
     * sqrt(T)) and moneyness (log forward moneyness of the strike less sigma^2 T / 2)
     * as above */
    double barrier_drift;     /* (r - q - sigma^2 / 2) T: terminal log return = drift + diffusion z */
    double barrier_distance;  /* |log(barrier / spot)| */
    double barrier_moneyness; /* log forward moneyness of the barrier less sigma^2 T / 2 */
    double rebate;            /* paid at expiry when the vanilla leg is not */
    double spot;
    double log_discount;      /* -r T */
    /* discretely observed barrier: steps hold drift = (r - q - sigma^2/2) t_i and
     * diffusion = sigma sqrt(t_i - t_{i-1}); event i holds knock_out = the noise level
     * sum(diffusion z) at which date i touches the barrier, coupon_barrier = T - t_i,
     * payment[0] = -r t_i, payment[1] = -r t_i - q (T - t_i), payment[2] = sqrt(T - t_i),
     * has_knock_out = 1 when date i is observed (the last step may be an unobserved
     * expiry).  moneyness, half_variance (sigma^2 / 2), strike, sign, rebate, spot and
     * log_discount as above. */
    double volatility;
    double dividend;
    /* continuous average (KGPU_PAYOFF_AVERAGE_*, asian.rs:374-1257), flat BSM rates, n
     * integration intervals.  strike, sign, spot and log_discount as above.
     * Arithmetic: growth += avg_drift + avg_width z per interval; the lead interval (if
     * any) draws avg_lead_drift + avg_lead_width z.  Geometric: distance = moneyness +
     * diffusion z with moneyness = initial moneyness + drift, diffusion = width and
     * log_scale = log width. */
    double avg_drift;             /* (r - q - sigma^2 / 2) dt */
    double avg_width;             /* sigma sqrt(dt) */
    double avg_lead_drift;        /* (r - q - sigma^2 / 2) lead */
    double avg_lead_width;        /* sigma sqrt(lead) */
    double avg_interval_forward;  /* (r - q) dt */
    double avg_weight;            /* future / period */
    double avg_log_spot;          /* ln(spot) */
    double avg_log_scale;         /* ln(spot) + ln(weight) */
    double avg_log_strike;        /* ln(strike) */
    double avg_fraction;          /* 1 / n: trapezoid weight of an interior fixing */
    double avg_half;              /* 0.5 / n: weight of the end fixings */
    double avg_log_fraction;      /* ln(1 / n) */
    double avg_log_half;          /* ln(0.5 / n) */
    double avg_rest;              /* 1 - 0.5 / n */
    double avg_log_rest;          /* ln(1 - 0.5 / n) */
    double avg_baseline;          /* weight ((spot - strike) / spot) */
    double control_log_strike;    /* geometric control (KGPU_C_AVERAGE_CONTROL) */
    double control_log_asset_scale;
    double control_first_weight;  /* 1 - 0.5 / n */
    double control_mean;          /* exact expected value of the control */
    /* continuous double barrier (KGPU_PAYOFF_DOUBLE_BARRIER): barrier_moneyness is the
     * lower barrier's terminal distance, so log(S_T / lower) = barrier_moneyness + noise;
     * strike, sign, diffusion, moneyness, barrier_drift, rebate, spot, log_discount as
     * for the single barrier */
    double band;                  /* log(upper / lower) */
    double band_initial;          /* log(spot / lower) */
    /* native delta / gamma samples (KGPU_C_OUTPUT_*) */
    double greek_log_spot;        /* ln(spot) */
    double greek_log_width;       /* digital: ln(sigma) + ln(sqrt(T)); arithmetic average:
                                     log width of an interval; geometric: log width */
    double greek_log_amount;      /* digital: ln(paid amount) */
    double greek_log_base_width;  /* geometric average: ln(sigma) + ln(sqrt(variance time)) */
    double greek_log_weight;      /* geometric average: ln(weight) */
    /* sampling dimensions per path: 0 = step_count x the model's normals per step.  A
     * larger value lays every path out over that many normals, so a contract whose grid
     * is a prefix of a longer one draws the longer grid's numbers (the lanes of a shared
     * daily grid, autocallable/portfolio.rs:1180-1190). */
    int32_t dimensions;
    int32_t reserved_tail;
} kgpu_contract;

/* A book of contracts sharing one model.  Arrays are indexed through the offsets in
 * each kgpu_contract; bridge_daily has one entry per grid step (may be NULL when no
 * contract uses KGPU_C_BRIDGE); events and intervals may be NULL when unused. */
typedef struct kgpu_book {
    int32_t contract_count;
    int32_t reserved;
    const kgpu_contract* contracts;
    int64_t step_total;
    const kgpu_step* steps;
    const uint8_t* step_flags;
    const kgpu_bridge_daily* bridge_daily;
    int32_t event_total;
    int32_t interval_total;
    const kgpu_event* events;
    const kgpu_bridge_interval* intervals;
} kgpu_book;

/* MonteCarloUncertaintyStatus (monte_carlo.rs:868-894). */
enum {
    KGPU_UNCERTAINTY_AVAILABLE = 0,
    KGPU_UNCERTAINTY_UNSUPPORTED_SAMPLING = 1,
    KGPU_UNCERTAINTY_INSUFFICIENT_OBSERVATIONS = 2,
    KGPU_UNCERTAINTY_INCOMPLETE_ANTITHETIC_PAIR = 3,
    KGPU_UNCERTAINTY_ZERO_OBSERVED_VARIANCE = 4
};

/* MonteCarloEstimate (monte_carlo.rs:858-865) per contract, plus GPU diagnostics. */
typedef struct kgpu_estimate {
    double price;
    double standard_error;       /* valid when status == KGPU_UNCERTAINTY_AVAILABLE */
    double sample_error;         /* i.i.d.-formula error, also reported for Sobol */
    int32_t uncertainty_status;  /* KGPU_UNCERTAINTY_* */
    int32_t reserved;
    uint64_t seed;
    double path_steps;           /* paths x grid steps represented by the estimate */
    double executed_steps;       /* grid steps actually simulated (early exits excluded) */
} kgpu_estimate;

typedef struct kgpu_context kgpu_context;

/* Creates a context on `device` (CUDA ordinal).  One context per thread, or serialise
 * calls on a shared context: a context owns one stream and its scratch buffers. */
kgpu_status kgpu_context_create(int device, kgpu_context** out);
void kgpu_context_destroy(kgpu_context* ctx);

/* The last error message recorded on `ctx` (thread-local when ctx is NULL). */
const char* kgpu_last_error_message(const kgpu_context* ctx);

/* Prices every contract of `book` under `model`.  `out` has book->contract_count
 * entries.  `cancel_flag` (may be NULL) is polled between launches and by persistent
 * kernels once per work item through host-mapped memory; a nonzero value ends the call
 * with KGPU_INTERRUPTED and no partial result (cancellation.rs:33-100).
 * The persistent schedules run their launch sequence (plan compilation, path kernel,
 * fixed-order reduction) as a CUDA graph once two consecutive calls on the context share
 * their model, settings, contract table and book arrays; the book's contents are read at
 * every launch, so a caller may change them between calls (see kgpu_context_last_graph).
 * Replaces PricingEngine::price_with_statistics of the MC engines and
 * MonteCarloAutocallableEngine::price_many (autocallable.rs:119-125). */
kgpu_status kgpu_price_book(kgpu_context* ctx, const kgpu_model* model, const kgpu_book* book,
                            const kgpu_settings* settings, kgpu_estimate* out,
                            const volatile int32_t* cancel_flag);

/* Device-resident variant for callers that keep plans in HBM and time the kernels
 * alone: `book` pointers are device pointers except `book->contracts` which is host;
 * the call stages nothing from the host beyond the contract table. */
kgpu_status kgpu_price_book_device(kgpu_context* ctx, const kgpu_model* model,
                                   const kgpu_book* device_book,
                                   const kgpu_settings* settings, kgpu_estimate* out);

/* Raw normal stream of one reference block: the `count` normals that block `block`
 * draws from Pcg32::new(seed, block) with Box-Muller (monte_carlo.rs:1678-1703,
 * 1830-1894), starting at normal index `first`.  precision selects FP64 or FP32
 * transforms.  Integer words are bit-exact; normals follow the precision. */
kgpu_status kgpu_pcg_normals(kgpu_context* ctx, uint64_t seed, uint64_t block, uint64_t first,
                             int64_t count, int32_t precision, double* out);

/* Raw PCG32 words of stream `stream` starting at word `first` (Pcg32::next, advance). */
kgpu_status kgpu_pcg_words(kgpu_context* ctx, uint64_t seed, uint64_t stream, uint64_t first,
                           int64_t count, uint32_t* out);

/* Scrambled Sobol integers (52-bit) for points [first, first+count) of `dimension`
 * out of `dimensions` (sobol.rs:85-174), and their inverse-normal transforms. */
kgpu_status kgpu_sobol_points(kgpu_context* ctx, uint64_t seed, int32_t dimensions,
                              int32_t dimension, uint64_t first, int64_t count,
                              uint64_t* bits_out, double* normals_out, int32_t precision);

/* ---------------------------------------------------------------------------------
 * American exercise by least-squares Monte Carlo (american.rs:955-1455).
 * --------------------------------------------------------------------------------- */
/* MLP: the polynomial basis plus a 3 -> 64 -> 64 -> 1 network fitted to what the
 * polynomial leaves unexplained.  MLP_STANDALONE: the network alone is the continuation
 * value, fitted to the in-the-money paths' discounted cash flows on the raw features
 * (log moneyness, variance, time). */
enum { KGPU_BASIS_QUADRATIC = 0, KGPU_BASIS_POLY3 = 1, KGPU_BASIS_MLP = 2, KGPU_BASIS_MLP_STANDALONE = 3 };

typedef struct kgpu_lsmc_settings {
    int32_t path_count;
    int32_t exercise_dates;    /* exercise intervals (step_count of the reference) */
    int32_t substeps;          /* Euler substeps per exercise interval (Heston) */
    int32_t basis;             /* KGPU_BASIS_* (QUADRATIC: BSM {1, S/K, (S/K)^2};
                                  POLY3: monomials of degree <= 3 in (S/K, v/theta)) */
    int32_t sampling;          /* KGPU_SAMPLING_PSEUDO_RANDOM */
    int32_t precision;         /* KGPU_PRECISION_*: path store and per-path arithmetic */
    int32_t mlp_epochs;        /* MLP basis: epochs per exercise date */
    int32_t mlp_batch;         /* MLP basis: minibatch size */
    int32_t mlp_hidden;        /* MLP basis: hidden width (64) */
    int32_t mlp_samples;       /* MLP basis: in-the-money samples trained on per date, the
                                  first ones in path order (0: all) */
    double mlp_learning_rate;
    uint64_t seed;
    uint64_t mlp_seed;
} kgpu_lsmc_settings;

typedef struct kgpu_lsmc_result {
    double price;              /* in-sample LSMC price, max(immediate, estimate) */
    double standard_error;     /* of the discounted cash flows */
    double out_of_sample;      /* lower bound on fresh paths, NaN when not requested */
    double out_of_sample_error;
    double wall_ms;            /* device time of the whole pricing */
    double path_store_ms;      /* forward pass writing the path store */
    double regression_ms;      /* backward regression / training */
} kgpu_lsmc_result;

/* Prices an American put or call (sign) with strike `strike` and expiry `expiry`
 * (years) under `model` (BSM or Heston).  `fresh_seed` != `settings.seed` also runs the
 * out-of-sample pass with the fitted exercise policy (american.rs:574-637). */
kgpu_status kgpu_lsmc_price(kgpu_context* ctx, const kgpu_model* model, double strike,
                            double sign, double expiry, const kgpu_lsmc_settings* settings,
                            uint64_t fresh_seed, kgpu_lsmc_result* out);

/* Prices the same American option in `count` (1..16) Black-Scholes-Merton scenarios --
 * the bumped contexts of the option's numerical Greeks -- with the quadratic basis, on
 * one set of paths: the scenarios share the seed's normals and the stored Brownian
 * coordinates, and each runs its own regression.  out[y] equals what kgpu_lsmc_price
 * returns for models[y] with the same settings, bit for bit.  Replaces the grouped
 * scenario pricing of MonteCarloVanillaEngine::greek_prices / american_spots
 * (crates/kiyosi/src/engines/monte_carlo/american.rs:820-946), which batches up to nine
 * contexts of one valuation date.  KGPU_UNSUPPORTED_OPERATION for Heston or local-vol
 * scenarios and for the other bases. */
kgpu_status kgpu_lsmc_price_scenarios(kgpu_context* ctx, const kgpu_model* models, int32_t count, double strike,
                                      double sign, double expiry, const kgpu_lsmc_settings* settings,
                                      uint64_t fresh_seed, kgpu_lsmc_result* out);

/* Prices contract `contract` of `device_book` without allocating device memory, for
 * callers that cannot call cudaMalloc (a host that reserves its device-memory budget up
 * front and hands out slices itself, a plugin inside such a host, or a latency-critical
 * loop that must never allocate).  It has no counterpart in the reference: kiyosi's CPU
 * engines own their buffers per call.
 *
 * All pointers of `device_book`, including `contracts`, are device pointers; `model`,
 * `settings` and `out` are host memory.  The call runs the FP64 plain schedule
 * (results equal kgpu_price_book's for the same plan and settings) on `stream` (a
 * cudaStream_t; NULL for the default stream), synchronises `stream` and returns when the
 * estimate is in `out`.  Before any launch it checks the contract as kgpu_price_book
 * checks a host book: step, event and bridge ranges, the event steps against the event
 * records and the order of the bridge intervals (read back through fixed host stack
 * buffers).  Limits: BSM or Heston models, pseudo-random sampling, settings asking for
 * KGPU_PRECISION_FP64 and KGPU_SCHEDULE_PLAIN (others are KGPU_UNSUPPORTED_OPERATION),
 * at most 4,194,304 samples per call.  Its scratch is one fixed 1.7 MB array in device
 * memory that every GPU loading this library holds until process exit.  The first call
 * on a device, with that device current, looks up the array's device address
 * (cudaGetSymbolAddress) and keeps it; make that first call before any stream capture.
 * The call synchronises `stream` before it returns.  Every call shares the array, so
 * calls that overlap on the GPU -- on different streams or from different threads --
 * race; serialise them.  Errors are reported through kgpu_last_error_message(NULL). */
kgpu_status kgpu_price_contract_noalloc(const kgpu_model* model, const kgpu_book* device_book,
                                        int32_t contract, const kgpu_settings* settings,
                                        kgpu_estimate* out, void* stream);

/* ---- Planning a book of notes on one shared daily grid (host code; no GPU) ----
 *
 * The host half of MonteCarloAutocallableEngine::price_many_on_shared_grid
 * (crates/kiyosi/src/engines/monte_carlo/autocallable.rs:127-152, planned by
 * autocallable/portfolio.rs): which notes join a shared daily grid (DailyGrids::prepare,
 * portfolio.rs:74-185), their groups (same_daily_grid, 872-901), the coupon families whose
 * interior members are interpolated (price_coupon_families, 570-667), and each group's
 * interval plan (SharedEvents::new, 903-1047) with one bridged lane contract per
 * simulated note.  Notes are given as flat terms; knock-in monitoring times and
 * observations are ranges of two shared tables. */

/* An autocallable note (AutocallableNote, crates/kiyosi/src/instruments/autocallable.rs).
 * Times are year fractions after valuation. */
enum {
    KGPU_NOTE_KNOCK_IN = 1,       /* knock_in_level is set */
    KGPU_NOTE_MONITORING = 2,     /* knock-in monitored on the listed times (else at expiry) */
    KGPU_NOTE_FIXED_COUPON = 4    /* knocked-in redemption is fixed_knock_in_coupon (else the
                                     capped downside) */
};
enum { KGPU_STATE_UNKNOWN = 0, KGPU_STATE_NO_EVENT = 1, KGPU_STATE_KNOCKED_IN = 2, KGPU_STATE_KNOCKED_OUT = 3 };

typedef struct kgpu_note {
    double initial_spot;
    double expiry;
    double knock_in_level;
    double upper_strike;
    double lower_strike;
    double maturity_coupon_rate;
    double period_coupon;
    double fixed_knock_in_coupon;
    double principal;
    double rebate_rate;
    double annual_rebate_rate;
    double effective_time;
    int32_t flags;               /* KGPU_NOTE_* */
    int32_t barrier_state;       /* KGPU_STATE_*: history strictly before valuation */
    int32_t observation_offset;  /* first kgpu_note_observation */
    int32_t observation_count;
    int32_t monitoring_offset;   /* first monitoring time (KGPU_NOTE_MONITORING) */
    int32_t monitoring_count;
} kgpu_note;

enum { KGPU_OBSERVATION_KNOCK_OUT = 1, KGPU_OBSERVATION_COUPON_BARRIER = 2 };

typedef struct kgpu_note_observation {
    double time;
    double knock_out_level;       /* KGPU_OBSERVATION_KNOCK_OUT */
    double coupon_barrier_level;  /* KGPU_OBSERVATION_COUPON_BARRIER */
    double coupon_rate;           /* annual coupon accrued on knock-out */
    int32_t flags;                /* KGPU_OBSERVATION_* */
    int32_t reserved;
} kgpu_note_observation;

typedef struct kgpu_shared_plan kgpu_shared_plan;

/* What a shared plan holds.  Pointers stay valid until kgpu_shared_plan_destroy. */
typedef struct kgpu_shared_plan_view {
    int32_t note_count;
    int32_t group_count;
    int32_t lane_count;                 /* simulated lanes of all groups */
    int32_t reserved;
    const int32_t* note_group;          /* [note_count]: the note's group, or -1 when the
                                           scalar engine quotes it */
    const int32_t* group_first_lane;    /* [group_count + 1]: group g's lanes are
                                           [group_first_lane[g], group_first_lane[g + 1]) */
    const int32_t* lane_note;           /* [lane_count]: the book index of each lane */
    const uint8_t* lane_fp32;           /* [lane_count]: the lane's plan is representable in
                                           FP32 (every finite nonzero value within
                                           [2^-100, 2^120]; the model is not checked) */
    const kgpu_book* group_books;       /* [group_count]: one book per group, its contracts
                                           the group's lanes in order, ready for
                                           kgpu_price_book with KGPU_SCHEDULE_SHARED_GRID */
    const int32_t* group_status;        /* [group_count]: KGPU_OK, or why the group's interval
                                           plan failed (raised when the group is priced) */
    const char* const* group_message;   /* [group_count]: the failure's message, or "" */
} kgpu_shared_plan_view;

/* Plans `note_count` notes under a BSM `model` (other models quote every note with the
 * scalar engine).  `simulate` (may be NULL) forces notes to be simulated although their
 * coupon family would interpolate them (the members whose interpolation cancelled).  A
 * note that fails the reference's checks (missing history, a non-finite plan) or that
 * needs no sampling is left to the scalar engine (note_group -1), whose planner reports
 * it.  KGPU_INVALID_INPUT for ranges outside the tables. */
kgpu_status kgpu_shared_plan_create(const kgpu_model* model, const kgpu_note* notes, int32_t note_count,
                                    const kgpu_note_observation* observations, int32_t observation_total,
                                    const double* monitoring, int32_t monitoring_total, const uint8_t* simulate,
                                    kgpu_shared_plan** out);

kgpu_status kgpu_shared_plan_get(const kgpu_shared_plan* plan, kgpu_shared_plan_view* out);

/* Fills the prices of the coupon families' interpolated members, linear in the coupon
 * between the family's lowest- and highest-coupon members (portfolio.rs:570-667).
 * note_prices[note_count] holds every simulated lane's price on entry.  retry[i] = 1
 * marks a member whose interpolation cancels (|price| < 1e-12 x the magnitude of its two
 * terms, or not finite), which the reference then simulates; its price is left as is. */
kgpu_status kgpu_shared_plan_interpolate(const kgpu_shared_plan* plan, double* note_prices, uint8_t* retry);

void kgpu_shared_plan_destroy(kgpu_shared_plan* plan);

/* Loss and parameter gradients of the LSMC continuation network on one batch, computed
 * by the tensor-core training kernel that the MLP basis of kgpu_lsmc_price runs (no
 * counterpart in the reference: exposed so the kernels' gradients can be checked).
 * params: KGPU_MLP_PARAMS floats, packed W1[64][3], b1[64], W2[64][64] (row = output
 * unit), b2[64], w3[64], b3; samples: count x 4 floats (three inputs, then the target).
 * grads receives d loss / d params of loss = mean((f(x) - target)^2); *loss that mean. */
#define KGPU_MLP_PARAMS 4481
kgpu_status kgpu_mlp_gradients(kgpu_context* ctx, const float* params, const float* samples, int32_t count,
                               float* grads, double* loss);

/* Trainers of the continuation network: 8-CTA thread-block clusters that keep the
 * network, the Adam state and the gradient sums on chip (what the network LSMC uses
 * where the device can co-schedule them), or one cooperative launch with two grid
 * barriers per step (the fallback). */
enum { KGPU_TRAINER_CLUSTER = 0, KGPU_TRAINER_GRID = 1 };

/* `steps` Adam steps (Kingma and Ba; beta1 0.9, beta2 0.999, eps 1e-8, zero initial
 * moments) of the tensor-core trainer `trainer` on `samples` (count x 4 floats, as for
 * kgpu_mlp_gradients), minibatch b being samples [b * batch, ...) cycled in order;
 * `params` (KGPU_MLP_PARAMS floats) is updated in place.  No counterpart in the
 * reference: exposed so the optimiser can be checked against a CPU restatement.  batch
 * <= 8192; KGPU_UNSUPPORTED_OPERATION when the device cannot run that trainer. */
kgpu_status kgpu_mlp_train(kgpu_context* ctx, float* params, const float* samples, int32_t count, int32_t batch,
                           int32_t steps, double learning_rate, int32_t trainer);

/* Instrumentation of the last call on `ctx`: device time from the first to the last
 * kernel of the call (CUDA events on the context's stream) and the number of kernel
 * launches it made. */
double kgpu_context_last_kernel_ms(const kgpu_context* ctx);
int32_t kgpu_context_last_launches(const kgpu_context* ctx);
/* Device time of the last pricing call's path kernels alone (the plain or persistent
 * kernel launches, without plan compilation and reductions), summed over launches. */
double kgpu_context_last_path_kernel_ms(const kgpu_context* ctx);
/* How the last kgpu_price_book call ran its launch sequence (no counterpart in the
 * reference): 0 launched directly, 1 captured into a CUDA graph and launched, 2 replayed
 * that graph.  The persistent schedules capture on the second of two consecutive calls
 * with the same model, settings, contract table and book arrays, and replay while the
 * calls keep them; any other call on the context drops the graph. */
int32_t kgpu_context_last_graph(const kgpu_context* ctx);

/* Throughput of the device's pipes, measured on `ctx`'s device (no counterpart in the
 * reference: the denominators of the benchmark's op-model roofline).  rates[0..4], in
 * thread operations per second: FP32 fused multiply-add, its packed two-lane form
 * (counted in FMAs), 32-bit logic (LOP3), the multi-function unit's base-2 logarithm,
 * and 32-bit loads that hit L1 with every lane of a warp at one address; entries past
 * the fifth are set to 0.  Runs about a
 * millisecond of kernels on the context's stream. */
kgpu_status kgpu_pipe_rates(kgpu_context* ctx, double* rates, int32_t count);

/* Library identification. */
int32_t kgpu_abi_version(void);
int32_t kgpu_device_count(void);

#ifdef __cplusplus
}
#endif

#endif /* KIYOSI_GB300_KGPU_H */
