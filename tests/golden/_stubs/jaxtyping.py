"""No-op stand-in for the ``jaxtyping`` annotations the reference imports.

Used only by ``make_golden.py`` to import the reference in a container where
``jaxtyping`` is not installed; every name is a subscriptable no-op type.
"""


class _NoOp:
    def __class_getitem__(cls, item):
        return cls


Float = Inexact = Shaped = Integer = Bool = Complex = Num = Int = _NoOp
