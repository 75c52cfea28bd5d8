"""kiyosi-gb300: GB300-native Monte Carlo and least-squares Monte Carlo engines for kiyosi.

The pricing path runs in libkiyosi_gpu.so (hand-written sm_103a CUDA behind the C ABI of
include/kgpu.h); this package is the Python host side that mirrors kiyosi's
`kiyosi.pricing.MonteCarlo*Engine` classes.  There is no CPU fallback: pricing raises
DeviceError when the CUDA library or a GPU is unavailable.
"""
from .errors import (ComputationFailureError, DeviceError, GreekUnavailableError,
                     InvalidInputError, KiyosiError, MissingHistoryError,
                     RootNotBracketedError, UnsupportedOperationError)
from .instruments import (CALL, PUT, Accumulator, AmericanOption, ArithmeticAveragePriceOption,
                          AsianOption, AutocallableNote, BarrierOption, DigitalOption,
                          EuropeanOption, GeometricAveragePriceOption, Observation,
                          PhoenixOption, SnowballOption)
from .market import (BlackScholesMertonParameters, HestonParameters, LocalVolatilitySurface,
                     PricingContext)

__all__ = [
    "Accumulator", "AmericanOption", "ArithmeticAveragePriceOption", "AsianOption",
    "AutocallableNote", "BarrierOption", "GeometricAveragePriceOption",
    "BlackScholesMertonParameters", "CALL", "ComputationFailureError", "DeviceError",
    "DigitalOption", "EuropeanOption", "GreekUnavailableError", "HestonParameters",
    "InvalidInputError", "KiyosiError", "LocalVolatilitySurface", "MissingHistoryError",
    "Observation", "PUT", "PhoenixOption", "PricingContext", "RootNotBracketedError",
    "SnowballOption", "UnsupportedOperationError",
]
