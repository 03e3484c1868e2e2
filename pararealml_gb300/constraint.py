"""Masked value constraints (host side).

Same contract as ``pararealml/constraint.py:6-131``: ``apply`` overwrites the
masked elements in place; ``multiply_and_add`` writes
``addend[mask] + multiplier * values`` (the Neumann ghost formula).  On the GPU
these become per-face value tables in which NaN marks an unmasked element.
"""

from __future__ import annotations

from typing import Optional, Sequence, Union

import numpy as np


class Constraint:
    def __init__(self, values: np.ndarray, mask: np.ndarray):
        if values.size != mask.sum():
            raise ValueError(
                f"number of values ({values.size}) must match number "
                f"of True elements in mask ({mask.sum()})"
            )
        self._values = np.array(values, copy=True)
        self._mask = np.array(mask, copy=True)
        self._values.setflags(write=False)
        self._mask.setflags(write=False)

    values = property(lambda self: self._values)
    mask = property(lambda self: self._mask)

    def apply(self, array: np.ndarray) -> np.ndarray:
        if array.shape[-self._mask.ndim:] != self._mask.shape:
            raise ValueError(
                f"input shape {array.shape} incompatible with mask shape {self._mask.shape}"
            )
        array[..., self._mask] = self._values
        return array

    def multiply_and_add(
        self, addend: np.ndarray, multiplier: Union[float, np.ndarray], result: np.ndarray
    ) -> np.ndarray:
        if addend.shape != result.shape:
            raise ValueError(
                f"addend shape {addend.shape} must match result shape {result.shape}"
            )
        if result.shape[-self._mask.ndim:] != self._mask.shape:
            raise ValueError(
                f"result shape {result.shape} incompatible with mask shape {self._mask.shape}"
            )
        if not isinstance(multiplier, float) and multiplier.shape != self._values.shape:
            raise ValueError(
                f"multiplier shape {multiplier.shape} must match values shape "
                f"{self._values.shape}"
            )
        result[..., self._mask] = addend[..., self._mask] + multiplier * self._values
        return result

    def dense(self) -> np.ndarray:
        """The constraint as a mask-shaped array with NaN where unmasked."""
        out = np.full(self._mask.shape, np.nan)
        out[self._mask] = self._values
        return out


def apply_constraints_along_last_axis(
    constraints: Optional[Union[Sequence[Optional[Constraint]], np.ndarray]],
    array: np.ndarray,
) -> np.ndarray:
    if constraints is not None:
        if array.ndim <= 1:
            raise ValueError(f"input dimensions ({array.ndim}) must be at least 2")
        if len(constraints) != array.shape[-1]:
            raise ValueError(
                f"number of constraints ({len(constraints)}) must match the "
                f"size of the input array's last axis ({array.shape[-1]})"
            )
        for i, c in enumerate(constraints):
            if c is not None:
                c.apply(array[..., i: i + 1])
    return array
