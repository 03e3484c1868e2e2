"""Learned operators mirroring ``pararealml.operators.ml`` (supervised)."""

from .supervised_ml_operator import SupervisedMLOperator, mean_squared_error, train_test_indices

__all__ = ["SupervisedMLOperator", "mean_squared_error", "train_test_indices"]
