"""Input types of the eigensubstitution path.

They mirror subby's own NamedTuples so that code written against
``subby.jax`` passes the same objects here:

* ``Tree`` — subby/formats.py:15-17 (re-exported by subby/jax/types.py:5):
  ``parentIndex`` (R,) int32 in preorder (``parentIndex[0] == -1``,
  ``parentIndex[n] < n``), ``distanceToParent`` (R,) float64.
* ``DiagModel`` — subby/jax/types.py:8-11: ``eigenvalues`` (A,),
  ``eigenvectors`` (A, A) with ``v[a, k]`` = component a of eigenvector k of
  the symmetrised rate matrix, ``pi`` (A,).
* ``IrrevDiagModel`` — subby/jax/types.py:14-18: complex ``eigenvalues``
  (A,), right eigenvectors ``eigenvectors`` V (A, A), ``eigenvectors_inv``
  V^-1 (A, A), real ``pi`` (A,) (root distribution).
* ``RateModel`` — subby/jax/types.py:21-23: ``subRate`` (A, A), ``rootProb``
  (A,); diagonalised on the host on entry (subby/jax/__init__.py:44-50).
"""
from __future__ import annotations

from typing import NamedTuple, Union

import numpy as np


class Tree(NamedTuple):
    parentIndex: np.ndarray
    distanceToParent: np.ndarray


class DiagModel(NamedTuple):
    eigenvalues: np.ndarray
    eigenvectors: np.ndarray
    pi: np.ndarray


class IrrevDiagModel(NamedTuple):
    eigenvalues: np.ndarray
    eigenvectors: np.ndarray
    eigenvectors_inv: np.ndarray
    pi: np.ndarray


class RateModel(NamedTuple):
    subRate: np.ndarray
    rootProb: np.ndarray


AnyDiagModel = Union[DiagModel, IrrevDiagModel]
AnyModel = Union[DiagModel, IrrevDiagModel, RateModel]
