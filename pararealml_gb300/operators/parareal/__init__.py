from .parareal_operator import FDMCoarsePropagator, PararealOperator
from .sharded import FDMSlicePropagator, SliceShardedParareal, slice_blocks

__all__ = ["PararealOperator", "FDMCoarsePropagator", "SliceShardedParareal", "FDMSlicePropagator", "slice_blocks"]
