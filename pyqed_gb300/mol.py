"""``Result`` container, field-for-field the reference's ``pyqed.mol.Result``
(``pyqed/mol.py:98-170``) so that code reading a reference result reads ours.

``times`` has Nt//nout + 1 entries starting at t0; ``observables`` and
``rholist`` are filled by the solver with the reference's row conventions.
"""
from __future__ import annotations

import pickle

import numpy as np

__all__ = ["Result", "load_result"]


class Result:
    def __init__(self, description=None, psi0=None, rho0=None, dt=None, Nt=None, times=None,
                 t0=0, nout=1):
        self.description = description
        self.dt = dt
        self.timesteps = self.nt = Nt
        self.observables = None
        self.rholist = None
        self.psilist = []
        self.psi = None
        self.rho0 = rho0
        self.psi0 = psi0
        self.nout = nout
        self.times = t0 + np.arange(Nt // nout + 1) * dt * nout

    def expect(self):
        return self.observables

    def dump(self, fname):
        """Pickle the result (``pyqed/mol.py:146-166``)."""
        with open(fname, "wb") as f:
            pickle.dump(self, f)

    def save(self, fname):
        self.dump(fname)


def load_result(fname):
    """Read a result saved with ``dump`` (``pyqed/mol.py:173-181``)."""
    with open(fname, "rb") as f:
        return pickle.load(f)
