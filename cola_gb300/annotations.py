"""Operator annotations (cola/annotations.py): PSD, SelfAdjoint, Unitary, Stiefel.

``PSD(op)`` returns a shallow copy of ``op`` carrying the annotation, as the reference's
``WrapMeta.__call__`` does (annotations.py:34-42).  Annotation inference for composites follows
``get_annotations`` (annotations.py:80-193): Kronecker / BlockDiag keep the intersection of their
factors, Sum drops Unitary/Stiefel, a Product with one non-scalar factor inherits it, and Identity
is Unitary and PSD.
"""
from __future__ import annotations

import copy
from functools import reduce


class WrapMeta(type):
    def __str__(cls):
        return cls.__name__

    def __repr__(cls):
        return cls.__name__

    def __call__(cls, obj):
        new_obj = copy.copy(obj)
        new_obj.annotations = set(obj.annotations) | {cls}
        new_obj.__dict__.pop("_lowered", None)
        return new_obj


class Annotation(metaclass=WrapMeta):
    pass


class SelfAdjoint(Annotation):
    """A^H = A (symmetric for real operators)."""


Hermitian = SelfAdjoint


class PSD(SelfAdjoint):
    """Positive semi-definite and self-adjoint."""


class Stiefel(Annotation):
    """A^H A = I."""


class Unitary(Stiefel):
    """A^H A = A A^H = I."""


def _intersect(ops):
    return reduce(lambda x, y: x & y, (set(op.annotations) for op in ops))


def get_annotations(A) -> set:
    from . import ops as O
    if isinstance(A, O.Identity):
        return {Unitary, PSD}
    if isinstance(A, (O.Kronecker, O.BlockDiag)):
        return _intersect(A.Ms)
    if isinstance(A, O.Sum):
        return _intersect(A.Ms) - {Unitary, Stiefel}
    if isinstance(A, O.Product):
        not_commuting = [M for M in A.Ms if not isinstance(M, O.ScalarMul)]
        if len(not_commuting) == 1:
            return set(not_commuting[0].annotations)
        return _intersect(A.Ms) & {Unitary, Stiefel}
    if isinstance(A, O.Transpose):
        return set(A.A.annotations)
    return set()


__all__ = ["Annotation", "SelfAdjoint", "Hermitian", "PSD", "Stiefel", "Unitary", "get_annotations"]
