"""Backends of the GPU hot path."""

from .dense import AssembledDense, DenseBackend, translation_basis

__all__ = ["AssembledDense", "DenseBackend", "translation_basis"]
