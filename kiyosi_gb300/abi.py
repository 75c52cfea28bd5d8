"""ctypes mirror of include/kgpu.h (the C ABI of libkiyosi_gpu.so).

Field order and types match the header exactly; `tests/test_abi.py` checks the struct
sizes against the compiled library.
"""
import ctypes as C

KGPU_OK = 0
KGPU_INVALID_INPUT = 1
KGPU_MISSING_HISTORY = 2
KGPU_UNSUPPORTED_OPERATION = 3
KGPU_GREEK_UNAVAILABLE = 4
KGPU_COMPUTATION_FAILURE = 5
KGPU_ROOT_NOT_BRACKETED = 6
KGPU_INTERRUPTED = 7
KGPU_DEVICE_ERROR = 8

SAMPLING_PSEUDO_RANDOM = 0
SAMPLING_SOBOL = 1
PRECISION_FP64 = 0
PRECISION_FP32 = 1
SCHEDULE_PLAIN = 0
SCHEDULE_PERSISTENT = 1
SCHEDULE_SHARED_GRID = 2
SCHEDULE_LANE_REFILL = 3

MODEL_BSM = 0
MODEL_HESTON = 1
MODEL_LOCAL_VOL = 2

PAYOFF_EUROPEAN = 0
PAYOFF_VANILLA_PATH = 1
PAYOFF_ASIAN = 2
PAYOFF_AUTOCALLABLE = 3
PAYOFF_ACCUMULATOR = 4
PAYOFF_DIGITAL = 5
PAYOFF_BARRIER = 6
PAYOFF_BARRIER_DISCRETE = 7
PAYOFF_AVERAGE_ARITHMETIC = 8
PAYOFF_AVERAGE_GEOMETRIC = 9
PAYOFF_DOUBLE_BARRIER = 10

STEP_KNOCK_IN = 1
STEP_EVENT = 2
STEP_FIXING = 4
STEP_ACCUMULATE = 8

C_HAS_KNOCK_IN = 1
C_KNOCKED_IN = 2
C_EXPIRY_KNOCK_IN = 4
C_DOWNSIDE = 8
C_BRIDGE = 16
C_ASSET_DIGITAL = 32
C_BARRIER_UP = 64
C_BARRIER_IN = 128
C_REBATE_AT_HIT = 256
C_CONDITION_ON_HIT = 512
C_CHECK_STEPS = 1024
C_AVERAGE_LEAD = 2048
C_AVERAGE_CONTROL = 4096
C_DOUBLE = 8192
C_OUTPUT_DELTA = 16384
C_OUTPUT_GAMMA = 32768

UNCERTAINTY_NAMES = {
    0: "available",
    1: "unsupported_sampling",
    2: "insufficient_observations",
    3: "incomplete_antithetic_pair",
    4: "zero_observed_variance",
}

BASIS_QUADRATIC = 0
BASIS_POLY3 = 1
BASIS_MLP = 2
BASIS_MLP_STANDALONE = 3
TRAINER_CLUSTER = 0
TRAINER_GRID = 1

_D = C.c_double
_I = C.c_int32
_P = C.POINTER


class Settings(C.Structure):
    _fields_ = [("path_count", _I), ("sampling", _I), ("antithetic", _I), ("precision", _I),
                ("schedule", _I), ("tile_paths", _I), ("ctas_per_sm", _I), ("refill", _I),
                ("seed", C.c_uint64)]


class Model(C.Structure):
    _fields_ = [("kind", _I), ("lv_time_count", _I), ("lv_spot_count", _I), ("reserved", _I),
                ("spot", _D), ("rate", _D), ("dividend", _D), ("volatility", _D),
                ("v0", _D), ("kappa", _D), ("theta", _D), ("xi", _D), ("rho", _D),
                ("lv_times", _P(_D)), ("lv_spots", _P(_D)), ("lv_values", _P(_D))]


class Step(C.Structure):
    _fields_ = [("drift", _D), ("diffusion", _D), ("time", _D), ("discount", _D)]


class Event(C.Structure):
    _fields_ = [("knock_out", _D), ("coupon_barrier", _D), ("payment", _D * 4),
                ("has_knock_out", _I), ("step", _I)]


class BridgeInterval(C.Structure):
    _fields_ = [("end", _I), ("reserved", _I), ("drift", _D), ("diffusion", _D)]


class BridgeDaily(C.Structure):
    _fields_ = [("weight", _D), ("width", _D)]


class Contract(C.Structure):
    _fields_ = [("payoff", _I), ("flags", _I), ("path_count", _I), ("step_count", _I),
                ("step_offset", C.c_int64), ("event_offset", _I), ("event_count", _I),
                ("bridge_offset", _I), ("bridge_count", _I),
                ("strike", _D), ("sign", _D),
                ("diffusion", _D), ("half_variance", _D), ("moneyness", _D), ("log_scale", _D),
                ("knock_in", _D), ("initial_cash", _D), ("terminal_base", _D),
                ("terminal_plain", _D), ("terminal_fixed", _D), ("downside_lower", _D),
                ("downside_upper", _D), ("downside_initial", _D), ("final_discount", _D),
                ("knock_out", _D), ("quantity", _D), ("daily_quantity", _D),
                ("acceleration", _D), ("log_strike", _D),
                ("barrier_drift", _D), ("barrier_distance", _D), ("barrier_moneyness", _D),
                ("rebate", _D), ("spot", _D), ("log_discount", _D), ("volatility", _D),
                ("dividend", _D), ("avg_drift", _D), ("avg_width", _D), ("avg_lead_drift", _D),
                ("avg_lead_width", _D), ("avg_interval_forward", _D), ("avg_weight", _D),
                ("avg_log_spot", _D), ("avg_log_scale", _D), ("avg_log_strike", _D), ("avg_fraction", _D),
                ("avg_half", _D), ("avg_log_fraction", _D), ("avg_log_half", _D),
                ("avg_rest", _D), ("avg_log_rest", _D), ("avg_baseline", _D),
                ("control_log_strike", _D), ("control_log_asset_scale", _D),
                ("control_first_weight", _D), ("control_mean", _D), ("band", _D),
                ("band_initial", _D), ("greek_log_spot", _D), ("greek_log_width", _D),
                ("greek_log_amount", _D), ("greek_log_base_width", _D), ("greek_log_weight", _D),
                ("dimensions", _I), ("reserved_tail", _I)]


class Book(C.Structure):
    _fields_ = [("contract_count", _I), ("reserved", _I), ("contracts", _P(Contract)),
                ("step_total", C.c_int64), ("steps", _P(Step)), ("step_flags", _P(C.c_uint8)),
                ("bridge_daily", _P(BridgeDaily)), ("event_total", _I), ("interval_total", _I),
                ("events", _P(Event)), ("intervals", _P(BridgeInterval))]


class Estimate(C.Structure):
    _fields_ = [("price", _D), ("standard_error", _D), ("sample_error", _D),
                ("uncertainty_status", _I), ("reserved", _I), ("seed", C.c_uint64),
                ("path_steps", _D), ("executed_steps", _D)]


class LsmcSettings(C.Structure):
    _fields_ = [("path_count", _I), ("exercise_dates", _I), ("substeps", _I), ("basis", _I),
                ("sampling", _I), ("precision", _I), ("mlp_epochs", _I), ("mlp_batch", _I),
                ("mlp_hidden", _I), ("mlp_samples", _I), ("mlp_learning_rate", _D),
                ("seed", C.c_uint64), ("mlp_seed", C.c_uint64)]


class LsmcResult(C.Structure):
    _fields_ = [("price", _D), ("standard_error", _D), ("out_of_sample", _D),
                ("out_of_sample_error", _D), ("wall_ms", _D), ("path_store_ms", _D),
                ("regression_ms", _D)]


NOTE_KNOCK_IN = 1
NOTE_MONITORING = 2
NOTE_FIXED_COUPON = 4
STATE_UNKNOWN = 0
STATE_NO_EVENT = 1
STATE_KNOCKED_IN = 2
STATE_KNOCKED_OUT = 3
OBSERVATION_KNOCK_OUT = 1
OBSERVATION_COUPON_BARRIER = 2


class Note(C.Structure):
    _fields_ = [("initial_spot", _D), ("expiry", _D), ("knock_in_level", _D), ("upper_strike", _D),
                ("lower_strike", _D), ("maturity_coupon_rate", _D), ("period_coupon", _D),
                ("fixed_knock_in_coupon", _D), ("principal", _D), ("rebate_rate", _D),
                ("annual_rebate_rate", _D), ("effective_time", _D), ("flags", _I),
                ("barrier_state", _I), ("observation_offset", _I), ("observation_count", _I),
                ("monitoring_offset", _I), ("monitoring_count", _I)]


class NoteObservation(C.Structure):
    _fields_ = [("time", _D), ("knock_out_level", _D), ("coupon_barrier_level", _D),
                ("coupon_rate", _D), ("flags", _I), ("reserved", _I)]


class SharedPlanView(C.Structure):
    _fields_ = [("note_count", _I), ("group_count", _I), ("lane_count", _I), ("reserved", _I),
                ("note_group", _P(_I)), ("group_first_lane", _P(_I)), ("lane_note", _P(_I)),
                ("lane_fp32", _P(C.c_uint8)), ("group_books", _P(Book)),
                ("group_status", _P(_I)), ("group_message", _P(C.c_char_p))]


STRUCT_SIZES = {
    "kgpu_settings": C.sizeof(Settings),
    "kgpu_model": C.sizeof(Model),
    "kgpu_step": C.sizeof(Step),
    "kgpu_event": C.sizeof(Event),
    "kgpu_bridge_interval": C.sizeof(BridgeInterval),
    "kgpu_bridge_daily": C.sizeof(BridgeDaily),
    "kgpu_contract": C.sizeof(Contract),
    "kgpu_book": C.sizeof(Book),
    "kgpu_estimate": C.sizeof(Estimate),
    "kgpu_lsmc_settings": C.sizeof(LsmcSettings),
    "kgpu_lsmc_result": C.sizeof(LsmcResult),
    "kgpu_note": C.sizeof(Note),
    "kgpu_note_observation": C.sizeof(NoteObservation),
    "kgpu_shared_plan_view": C.sizeof(SharedPlanView),
}

# Every entry point include/kgpu.h declares.
EXPORTED_SYMBOLS = (
    "kgpu_context_create", "kgpu_context_destroy", "kgpu_last_error_message",
    "kgpu_price_book", "kgpu_price_book_device", "kgpu_pcg_normals", "kgpu_pcg_words",
    "kgpu_sobol_points", "kgpu_lsmc_price", "kgpu_context_last_kernel_ms",
    "kgpu_context_last_path_kernel_ms",
    "kgpu_context_last_launches", "kgpu_abi_version", "kgpu_device_count", "kgpu_pipe_rates",
    "kgpu_price_contract_noalloc", "kgpu_mlp_gradients", "kgpu_mlp_train", "kgpu_lsmc_price_scenarios",
    "kgpu_shared_plan_create", "kgpu_shared_plan_get", "kgpu_shared_plan_interpolate",
    "kgpu_shared_plan_destroy", "kgpu_context_last_graph",
)
MLP_PARAMS = 4481


def declare(lib):
    """Declares argument and result types of every kgpu_* entry point on `lib`."""
    V = C.c_void_p
    lib.kgpu_context_create.argtypes = [C.c_int, _P(V)]
    lib.kgpu_context_create.restype = _I
    lib.kgpu_context_destroy.argtypes = [V]
    lib.kgpu_context_destroy.restype = None
    lib.kgpu_last_error_message.argtypes = [V]
    lib.kgpu_last_error_message.restype = C.c_char_p
    lib.kgpu_price_book.argtypes = [V, _P(Model), _P(Book), _P(Settings), _P(Estimate),
                                    _P(_I)]
    lib.kgpu_price_book.restype = _I
    lib.kgpu_price_book_device.argtypes = [V, _P(Model), _P(Book), _P(Settings), _P(Estimate)]
    lib.kgpu_price_book_device.restype = _I
    lib.kgpu_pcg_normals.argtypes = [V, C.c_uint64, C.c_uint64, C.c_uint64, C.c_int64, _I,
                                     _P(_D)]
    lib.kgpu_pcg_normals.restype = _I
    lib.kgpu_pcg_words.argtypes = [V, C.c_uint64, C.c_uint64, C.c_uint64, C.c_int64,
                                   _P(C.c_uint32)]
    lib.kgpu_pcg_words.restype = _I
    lib.kgpu_sobol_points.argtypes = [V, C.c_uint64, _I, _I, C.c_uint64, C.c_int64,
                                      _P(C.c_uint64), _P(_D), _I]
    lib.kgpu_sobol_points.restype = _I
    lib.kgpu_lsmc_price.argtypes = [V, _P(Model), _D, _D, _D, _P(LsmcSettings), C.c_uint64,
                                    _P(LsmcResult)]
    lib.kgpu_lsmc_price.restype = _I
    lib.kgpu_lsmc_price_scenarios.argtypes = [V, _P(Model), _I, _D, _D, _D, _P(LsmcSettings), C.c_uint64,
                                              _P(LsmcResult)]
    lib.kgpu_lsmc_price_scenarios.restype = _I
    lib.kgpu_context_last_kernel_ms.argtypes = [V]
    lib.kgpu_context_last_kernel_ms.restype = C.c_double
    lib.kgpu_context_last_path_kernel_ms.argtypes = [V]
    lib.kgpu_context_last_path_kernel_ms.restype = C.c_double
    lib.kgpu_context_last_launches.argtypes = [V]
    lib.kgpu_context_last_launches.restype = _I
    lib.kgpu_context_last_graph.argtypes = [V]
    lib.kgpu_context_last_graph.restype = _I
    lib.kgpu_price_contract_noalloc.argtypes = [_P(Model), _P(Book), _I, _P(Settings),
                                                _P(Estimate), V]
    lib.kgpu_price_contract_noalloc.restype = _I
    lib.kgpu_mlp_gradients.argtypes = [V, _P(C.c_float), _P(C.c_float), _I, _P(C.c_float),
                                       _P(_D)]
    lib.kgpu_mlp_gradients.restype = _I
    lib.kgpu_abi_version.argtypes = []
    lib.kgpu_abi_version.restype = _I
    lib.kgpu_device_count.argtypes = []
    lib.kgpu_device_count.restype = _I
    lib.kgpu_mlp_train.argtypes = [V, C.POINTER(C.c_float), C.POINTER(C.c_float), _I, _I, _I, _D, _I]
    lib.kgpu_mlp_train.restype = _I
    lib.kgpu_pipe_rates.argtypes = [V, C.POINTER(_D), _I]
    lib.kgpu_pipe_rates.restype = _I
    lib.kgpu_shared_plan_create.argtypes = [_P(Model), _P(Note), _I, _P(NoteObservation), _I, _P(_D), _I,
                                            _P(C.c_uint8), _P(V)]
    lib.kgpu_shared_plan_create.restype = _I
    lib.kgpu_shared_plan_get.argtypes = [V, _P(SharedPlanView)]
    lib.kgpu_shared_plan_get.restype = _I
    lib.kgpu_shared_plan_interpolate.argtypes = [V, _P(_D), _P(C.c_uint8)]
    lib.kgpu_shared_plan_interpolate.restype = _I
    lib.kgpu_shared_plan_destroy.argtypes = [V]
    lib.kgpu_shared_plan_destroy.restype = None
    return lib
