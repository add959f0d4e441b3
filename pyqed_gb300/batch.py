"""Batched entry points: many independent instances of uneven dimension in
one launch.

``propagate_batch`` generalises the reference's single-instance loops
(``_lindblad``, ``pyqed/oqs.py:1596-1696``; ``_lindblad_driven``,
``pyqed/oqs.py:1699-1806``) to a list of instances; ``correlation_batch``
is the reference's quantum-regression correlation ``<A(t) B>``
(``_correlation_2p_1t``, ``pyqed/oqs.py:717-791``) for a list of instances,
with the observable accumulated in FP64 on the GPU.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _capi as C
from .engine import Propagator, diagonal_of, pack, to_dense

__all__ = ["propagate_batch", "correlation_batch", "BatchInputs", "prepare_batch"]


class BatchInputs:
    """Packed host arrays of a batch (complex128) and its engine arguments."""

    def __init__(self, dims, H, cops, cops_kind, n_cops, rho0, eops, n_eops, dops=None,
                 n_drive=0):
        self.dims, self.H, self.cops, self.cops_kind, self.n_cops = dims, H, cops, cops_kind, n_cops
        self.rho0, self.eops, self.n_eops, self.dops, self.n_drive = rho0, eops, n_eops, dops, n_drive

    def nbytes(self):
        return sum(a.nbytes for a in (self.H, self.cops, self.rho0, self.eops, self.dops)
                   if a is not None)


def prepare_batch(H, c_ops, rho0, e_ops=None, drive_ops=None):
    """Lists per instance -> ``BatchInputs`` (packed layout of the C ABI).

    c_ops[b] is a list of K operators (dense or scipy.sparse) or, when every
    operator of every instance is diagonal, they are passed as diagonals.
    drive_ops[b] is a list of the H_i of H(t) = H0 - sum_i f_i(t) H_i.
    """
    n = len(H)
    Hd = [to_dense(h) for h in H]
    dims = np.array([h.shape[0] for h in Hd], dtype=np.int32)
    # Instances may carry different numbers of collapse operators; the packed
    # layout has K = max per instance, padded with zero operators (which add
    # nothing to the RHS).
    c_ops = [list(c or []) for c in c_ops]
    K = max(len(c) for c in c_ops)
    kind, cops = "none", None
    if K:
        diags = [[diagonal_of(c) for c in cl] for cl in c_ops]
        if all(d is not None for dl in diags for d in dl):
            kind = "diag"
            cops = pack([np.concatenate([np.stack(dl) if dl else np.zeros((0, dims[b]), complex),
                                         np.zeros((K - len(dl), dims[b]), complex)])
                         for b, dl in enumerate(diags)])
        else:
            kind = "dense"
            cops = pack([to_dense(c) for cl in c_ops for c in cl] if len({len(c) for c in c_ops}) == 1
                        else [np.concatenate([np.stack([to_dense(c) for c in cl]) if cl else
                                              np.zeros((0, dims[b], dims[b]), complex),
                                              np.zeros((K - len(cl), dims[b], dims[b]), complex)])
                              for b, cl in enumerate(c_ops)])
    E = 0
    eops = None
    if e_ops is not None:
        Es = {len(e) for e in e_ops}
        if len(Es) != 1:
            raise ValueError("every instance needs the same number of observables")
        E = Es.pop()
        eops = pack([to_dense(e) for el in e_ops for e in el]) if E else None
    D, dops = 0, None
    if drive_ops is not None:
        D = len(drive_ops[0])
        dops = pack([to_dense(h) for hl in drive_ops for h in hl])
    r0 = pack([to_dense(r) for r in rho0])
    for b in range(n):
        if to_dense(rho0[b]).shape != (dims[b], dims[b]):
            raise ValueError("rho0[%d] does not match H[%d]" % (b, b))
    return BatchInputs(dims, pack(Hd), cops, kind, K, r0, eops, E, dops, D)


def _select(shard, H, c_ops, rho0, e_ops, drive_ops, drive):
    """This rank's instances of a batch (``pyqed_gb300.shard``); returns the
    indices and the per-instance arguments restricted to them."""
    from .shard import resolve_shard, shard_indices, take
    rank, world = resolve_shard(shard)
    dims = [to_dense(h).shape[0] for h in H]
    idx = shard_indices(dims, rank, world)
    if drive is not None:
        drive = np.asarray(drive, dtype=np.float64)
        if drive.ndim == 3:  # per-instance samples
            drive = drive[idx]
    return (idx, take(H, idx), take(c_ops, idx), take(rho0, idx), take(e_ops, idx),
            take(drive_ops, idx), drive)


def propagate_batch(H, c_ops, rho0, dt, Nt, e_ops=None, *, obs_t0=True, store_every=0,
                    precision="fp32", schedule="auto", drive_ops=None, drive=None,
                    device=None, return_rho=True, shard=None, check=None):
    """Propagate a batch; returns dict(observables (n, rows, E), rho list,
    states list, info).  ``schedule``: "auto", "cta", "gemm" or "tune" (the
    autotuner times the candidates first, see ``pyqed_gb300.autotune``).

    ``shard=(rank, world_size)`` (or ``"dist"``: the torch.distributed ranks)
    propagates only this rank's share of the instances (greedy balance of
    N^3, ``pyqed_gb300.shard.partition``) on this process's GPU; the result
    then holds those instances, in batch order, and ``indices`` their
    positions in the batch (``pyqed_gb300.shard.gather`` reassembles).

    ``check=tol`` runs the per-step FP64 check of every instance's trace and
    (for a Hermitian rho0) hermiticity at that tolerance; ``check`` in the
    result holds the largest deviations per instance and ``check_flags``
    whether each stayed within the tolerance (a RuntimeWarning names the
    instances that did not)."""
    idx = None
    if shard is not None:
        idx, H, c_ops, rho0, e_ops, drive_ops, drive = _select(shard, H, c_ops, rho0, e_ops,
                                                               drive_ops, drive)
        if len(idx) == 0:
            E = len(e_ops[0]) if e_ops else 0
            return dict(info=None, indices=idx, observables=np.zeros((0, Nt + int(obs_t0), E), complex),
                        rho=[] if return_rho else None, states=[] if store_every > 0 else None)
    bi = prepare_batch(H, c_ops, rho0, e_ops, drive_ops)
    drive_shared = True
    if bi.n_drive:
        drive = np.asarray(drive, dtype=np.float64)
        drive_shared = drive.ndim == 2
    options = {}
    tuned = None
    if schedule == "tune":
        from .autotune import tune
        tuned = tune(bi, dt=dt, precision=precision, obs_t0=obs_t0, drive=drive,
                     drive_shared=drive_shared, device=device)
        schedule, options = tuned["schedule"], tuned["options"]
    prop = Propagator(bi.dims, nt=Nt, dt=dt, n_cops=bi.n_cops, cops_kind=bi.cops_kind,
                      n_eops=bi.n_eops, n_drive=bi.n_drive, obs_t0=obs_t0,
                      store_every=store_every, precision=precision, schedule=schedule,
                      drive_shared=drive_shared, device=device)
    try:
        for k, v in options.items():
            prop.set_option(k, v)
        if check:
            prop.set_check(check)
        prop.set_operators(bi.H, bi.cops, bi.eops, bi.dops)
        d = torch.from_numpy(drive.ravel()).to(prop.device) if bi.n_drive else None
        out = prop.alloc_outputs(want_obs=True, want_rho=return_rho,
                                 want_states=store_every > 0)
        obs, rho, st = prop.propagate_device(prop.to_device(bi.rho0), d, out)
        flags = prop.check_errors()
        res = dict(info=prop.info())
        if check:
            res["check"] = prop.check_stats()
            res["check_flags"] = flags == C.LGB_OK
        if tuned is not None:
            res["tuned"] = tuned
        res["observables"] = (prop.unpack_obs(obs) if obs is not None
                              else np.zeros((prop.n_inst, Nt + int(obs_t0), 0), complex))
        res["rho"] = prop.unpack_rho(rho) if rho is not None else None
        res["states"] = prop.unpack_states(st) if st is not None else None
        if idx is not None:
            res["indices"] = idx
    finally:
        prop.close()
    return res


def correlation_batch(H, c_ops, rho0, a_ops, b_ops, dt, Nt, *, precision="fp32",
                      schedule="auto", device=None, shard=None):
    """C_b(t_k) = Tr[A_b rho_b(t_k)], rho_b(0) = B_b rho0_b, k = 1..Nt.

    Returns an (n_inst, Nt) complex128 array.  With ``shard`` (see
    ``propagate_batch``) only this rank's instances are propagated and the
    result is ``(indices, C)`` with C of shape (len(indices), Nt).
    """
    idx = None
    if shard is not None:
        idx, H, c_ops, rho0, _, _, _ = _select(shard, H, c_ops, rho0, None, None, None)
        a_ops, b_ops = [a_ops[int(b)] for b in idx], [b_ops[int(b)] for b in idx]
        if len(idx) == 0:
            return idx, np.zeros((0, Nt), complex)
    seeds = [to_dense(b) @ to_dense(r) for b, r in zip(b_ops, rho0)]
    res = propagate_batch(H, c_ops, seeds, dt, Nt, e_ops=[[a] for a in a_ops], obs_t0=False,
                          precision=precision, schedule=schedule, device=device,
                          return_rho=False)
    C_ = res["observables"][:, :, 0]
    return C_ if idx is None else (idx, C_)
