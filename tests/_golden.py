"""Loader for the golden fixtures produced by tests/golden/make_golden.py."""
import glob
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(__file__), "golden")


def names():
    return sorted(os.path.splitext(os.path.basename(p))[0]
                  for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def load(name):
    with np.load(os.path.join(GOLDEN_DIR, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def model_dict(g):
    """The fixture's model as the oracle's dict (irreversible when it
    carries eigenvectors_inv)."""
    m = {'eigenvalues': g['eigenvalues'], 'eigenvectors': g['eigenvectors'], 'pi': g['pi']}
    if 'eigenvectors_inv' in g:
        m['eigenvectors_inv'] = g['eigenvectors_inv']
        m['reversible'] = False
    return m
