"""Exception classes mirroring kiyosi's Python error mapping (kiyosi-python/src/error.rs:4-30).

Status codes of the C ABI (include/kgpu.h) map one-to-one onto these classes.
"""


class KiyosiError(Exception):
    """Base class of kiyosi errors."""


class InvalidInputError(KiyosiError, ValueError):
    pass


class MissingHistoryError(KiyosiError):
    pass


class UnsupportedOperationError(KiyosiError):
    pass


class GreekUnavailableError(KiyosiError):
    pass


class ComputationFailureError(KiyosiError, ArithmeticError):
    pass


class RootNotBracketedError(KiyosiError):
    pass


class DeviceError(KiyosiError, RuntimeError):
    """The GPU failed (no device, out of memory, launch failure)."""


def raise_for_status(status: int, message: str = "") -> None:
    if status == 0:
        return
    if status == 7:
        # Error::Io(Interrupted) from cancellation maps to OSError in kiyosi.
        raise InterruptedError(message or "Monte Carlo pricing was cancelled")
    cls = {
        1: InvalidInputError,
        2: MissingHistoryError,
        3: UnsupportedOperationError,
        4: GreekUnavailableError,
        5: ComputationFailureError,
        6: RootNotBracketedError,
        8: DeviceError,
    }.get(status, KiyosiError)
    raise cls(message or f"kgpu status {status}")
