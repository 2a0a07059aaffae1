"""Pauli-sum representations used by the SQD path."""
from .symplectic import PauliSumXZ

__all__ = ['PauliSumXZ']
