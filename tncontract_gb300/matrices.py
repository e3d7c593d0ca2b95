"""Frequently used single-site operators: the drop-in for
tncontract/matrices.py.  Host ``numpy.matrix`` values, as the reference
returns; pass them to ``Tensor`` to move them to the device."""
from __future__ import annotations

import numpy as np

__all__ = ['sigmap', 'sigmam', 'sigmax', 'sigmay', 'sigmaz', 'destroy', 'create', 'identity', 'basis']


def sigmap():
    """Raising operator |0><1| of a spin 1/2 (``matrices.py:17-18``)."""
    m = np.zeros((2, 2))
    m[0, 1] = 1.0
    return np.matrix(m)


def sigmam():
    """Lowering operator |1><0| (``matrices.py:21-22``)."""
    return sigmap().T


def sigmax():
    return np.matrix([[0.0, 1.0], [1.0, 0.0]])


def sigmay():
    return np.matrix([[0.0, -1j], [1j, 0.0]])


def sigmaz():
    return np.matrix(np.diag([1.0, -1.0]))


def destroy(dim):
    """Annihilation operator on ``dim`` levels: sqrt(n) on the first
    superdiagonal (``matrices.py:37-46``)."""
    return np.matrix(np.diag(np.sqrt(np.arange(1, dim)), 1))


def create(dim):
    """Creation operator, the adjoint of ``destroy`` (``matrices.py:49-58``)."""
    return destroy(dim).H


def identity(dim):
    return np.matrix(np.eye(dim))


def basis(dim, i):
    """Column vector e_i of length ``dim`` (``matrices.py:74-80``)."""
    v = np.zeros((dim, 1))
    v[i, 0] = 1.0
    return np.matrix(v)
