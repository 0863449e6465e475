"""Exceptions raised by the host layer, named after the Julia exceptions the reference throws."""


class DimensionMismatch(Exception):
    """Sizes of the operands do not agree (Julia's ``DimensionMismatch``)."""


class ArgumentError(ValueError):
    """An argument is invalid or unsupported (Julia's ``ArgumentError``)."""
