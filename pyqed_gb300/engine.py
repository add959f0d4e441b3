"""Host-side engine: packs batches, owns a C-ABI plan, runs propagations.

``Propagator`` is the one object between the reference-shaped Python API
(``pyqed_gb300.oqs``) and the CUDA library.  Device memory, streams and
pinned host buffers come from PyTorch; the arithmetic runs in the library's
kernels.  There is no CPU fallback: without a CUDA device the constructor
raises.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _capi as C

__all__ = ["Propagator", "pack", "to_dense", "diagonal_of"]


def to_dense(a):
    """numpy / scipy.sparse / torch -> complex128 numpy array."""
    if a is None:
        return None
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    if hasattr(a, "toarray"):
        a = a.toarray()
    return np.ascontiguousarray(np.asarray(a, dtype=np.complex128))


def diagonal_of(a):
    """Diagonal of ``a`` if ``a`` is diagonal, else None."""
    if hasattr(a, "tocoo"):
        coo = a.tocoo()
        if np.any(coo.row != coo.col):
            return None
        d = np.zeros(a.shape[0], complex)
        np.add.at(d, coo.row, coo.data)
        return d
    m = to_dense(a)
    d = np.diag(m).copy()
    if np.count_nonzero(m - np.diag(d)):
        return None
    return d


def pack(mats):
    """Concatenate row-major complex128 matrices (the packed layout)."""
    if len(mats) == 0:
        return np.zeros(0, np.complex128)
    return np.concatenate([np.ascontiguousarray(m, dtype=np.complex128).ravel() for m in mats])


def _device(device):
    if not torch.cuda.is_available():
        raise RuntimeError("pyqed_gb300 needs a CUDA device (no CPU fallback)")
    return torch.device(device if device is not None else "cuda")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() > 0 else None


class Propagator:
    """A batch of independent Lindblad instances on one GPU.

    dims      instance dimensions (length n_inst)
    n_cops    collapse operators per instance; ``cops_kind`` 'dense' or 'diag'
    n_eops    observables per instance
    n_drive   drive terms, H(t) = H0 - sum_i f_i(t) H_i
    obs_t0    observable row 0 at t0 (static ``run`` convention)
    """

    def __init__(self, dims, *, nt, dt, n_cops=0, cops_kind="none", n_eops=0, n_drive=0,
                 obs_t0=False, store_every=0, precision="fp32", schedule="auto",
                 drive_shared=True, device=None, flags=0, checkpoint_every=0):
        self.device = _device(device)
        self.dims = np.asarray(dims, dtype=np.int32)
        self.n_inst = int(self.dims.size)
        self.nt, self.dt = int(nt), float(dt)
        self.n_cops, self.n_eops, self.n_drive = int(n_cops), int(n_eops), int(n_drive)
        self.cops_kind = {"none": C.COPS_NONE, "dense": C.COPS_DENSE, "diag": C.COPS_DIAG}[
            cops_kind if self.n_cops else "none"]
        self.obs_t0 = bool(obs_t0)
        self.store_every = int(store_every)
        self.precision = precision
        self.drive_shared = bool(drive_shared)
        self.off = np.concatenate([[0], np.cumsum(self.dims.astype(np.int64) ** 2)])
        self.doff = np.concatenate([[0], np.cumsum(self.dims.astype(np.int64))])
        self.n_store = self.nt // self.store_every if self.store_every > 0 else 0
        prob = C.Problem(
            n_inst=self.n_inst, n_cops=self.n_cops, cops_kind=self.cops_kind,
            n_eops=self.n_eops, n_drive=self.n_drive, nt=self.nt, obs_t0=int(self.obs_t0),
            store_every=self.store_every, precision=C.PREC[precision],
            schedule=C.SCHED[schedule], drive_shared=int(self.drive_shared), flags=int(flags),
            dt=self.dt, checkpoint_every=int(checkpoint_every), reserved=0)
        self._lib = C.lib()
        self._plan = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            dims_c = (ctypes.c_int32 * self.n_inst)(*self.dims.tolist())
            C.check(self._lib.lgb_plan_create(ctypes.byref(self._plan), ctypes.byref(prob), dims_c),
                    "lgb_plan_create")
        self._keep = []

    # -- lifetime -----------------------------------------------------------
    def close(self):
        if getattr(self, "_plan", None) is not None and self._plan.value:
            self._lib.lgb_plan_destroy(self._plan)
            self._plan = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_option(self, name, value):
        """Option of the plan (``lgb_plan_set_option``): ``tc_pairs`` (0/1),
        ``gemm_waves`` (1/2), ``gemm_ksplit`` (split-K cap), ``graph_steps``
        (RK4 steps per CUDA graph), ``gemm_persist`` (0/1: the persistent
        split-precision kernel for 64 < N <= 256), ``check`` (0 off, v: the
        per-step trace and hermiticity check at tolerance 10^-v), or the
        error-path test hook ``test_stall`` (0/1)."""
        C.check(self._lib.lgb_plan_set_option(self._plan, C.OPT[name], int(value)),
                "lgb_plan_set_option")

    def set_check(self, tol):
        """Per-step FP64 check of trace and hermiticity at tolerance ``tol``
        (rounded to a power of ten, 1e-1 .. 1e-15); None or 0 turns it off."""
        if not tol:
            self.set_option("check", 0)
            return
        v = int(round(-np.log10(float(tol))))
        if not 1 <= v <= 15:
            raise ValueError("check tolerance must lie in [1e-15, 1e-1]")
        self.set_option("check", v)

    def check_stats(self):
        """(n_inst, 2) array of the last propagate's largest |Tr rho(t) -
        Tr rho0| and max_ij |rho_ij - conj(rho_ji)| (-1: rho0 not Hermitian,
        hermiticity not checked)."""
        buf = (ctypes.c_double * (2 * self.n_inst))()
        C.check(self._lib.lgb_plan_check_stats(self._plan, buf), "lgb_plan_check_stats")
        return np.array(buf[:], dtype=np.float64).reshape(self.n_inst, 2)

    def info(self):
        inf = C.PlanInfo()
        C.check(self._lib.lgb_plan_get_info(self._plan, ctypes.byref(inf)), "lgb_plan_get_info")
        return dict(schedule=C.SCHED_NAME[inf.schedule], precision=C.PREC_NAME[inf.precision],
                    smem_bytes=inf.smem_bytes, launches=inf.launches_per_propagate,
                    workspace_bytes=inf.workspace_bytes, flops_per_step=inf.flops_per_step,
                    persistent_instances=inf.persistent_instances)

    # -- helpers ---------------------------------------------------------------
    def to_device(self, host, pin=False):
        """complex128 numpy (packed) -> device tensor."""
        t = torch.from_numpy(np.ascontiguousarray(host, dtype=np.complex128))
        if pin:
            t = t.pin_memory()
        return t.to(self.device, non_blocking=pin)

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    # -- operators -------------------------------------------------------------
    def set_operators(self, H, cops=None, eops=None, dops=None):
        """Device tensors (packed complex128) or numpy arrays (uploaded)."""
        def dev(x):
            if x is None:
                return None
            if isinstance(x, torch.Tensor):
                return x.to(self.device)
            return self.to_device(x)
        H, cops, eops, dops = dev(H), dev(cops), dev(eops), dev(dops)
        self._keep = [H, cops, eops, dops]
        with torch.cuda.device(self.device):
            C.check(self._lib.lgb_plan_set_operators(self._plan, _ptr(H), _ptr(cops), _ptr(eops),
                                                     _ptr(dops), self._stream()),
                    "lgb_plan_set_operators")

    # -- propagation -----------------------------------------------------------------
    def alloc_outputs(self, want_obs=True, want_rho=True, want_states=False):
        nrows = self.nt + int(self.obs_t0)
        z = lambda n: torch.empty(int(n), dtype=torch.complex128, device=self.device)  # noqa: E731
        obs = z(self.n_inst * nrows * self.n_eops) if (want_obs and self.n_eops) else None
        rho = z(self.off[-1]) if want_rho else None
        st = z(self.n_store * self.off[-1]) if (want_states and self.n_store) else None
        return obs, rho, st

    def propagate_device(self, rho0, drive=None, out=None):
        """rho0: device complex128 (packed); drive: device float64 or None.
        Returns (obs, rho, states) device tensors (None where not requested)."""
        obs, rho, st = out if out is not None else self.alloc_outputs()
        with torch.cuda.device(self.device):
            C.check(self._lib.lgb_plan_propagate(self._plan, _ptr(rho0), _ptr(drive), _ptr(obs),
                                                 _ptr(rho), _ptr(st), self._stream()),
                    "lgb_plan_propagate")
        return obs, rho, st

    def errors(self):
        flags = (ctypes.c_int32 * self.n_inst)()
        self._lib.lgb_plan_errors(self._plan, flags)
        return np.array(flags[:], dtype=np.int32)

    def check_errors(self):
        """Raise on the first failed instance; instances that only failed the
        per-step check (their outputs are complete) give a RuntimeWarning.
        Returns the per-instance flags."""
        f = self.errors()
        bad = np.nonzero((f != C.LGB_OK) & (f != C.LGB_ERR_CHECK))[0]
        if bad.size:
            raise C.LindbladError(int(f[bad[0]]), "instance %d" % int(bad[0]))
        flagged = np.nonzero(f == C.LGB_ERR_CHECK)[0]
        if flagged.size:
            import warnings
            warnings.warn("%d instance(s) exceeded the per-step trace/hermiticity check "
                          "tolerance (first: %d)" % (flagged.size, int(flagged[0])), RuntimeWarning,
                          stacklevel=2)
        return f

    # -- unpacking -------------------------------------------------------------------
    def unpack_obs(self, obs):
        nrows = self.nt + int(self.obs_t0)
        return obs.cpu().numpy().reshape(self.n_inst, nrows, self.n_eops)

    def unpack_rho(self, rho):
        h = rho.cpu().numpy()
        return [h[self.off[b]:self.off[b + 1]].reshape(self.dims[b], self.dims[b])
                for b in range(self.n_inst)]

    def unpack_states(self, st):
        h = st.cpu().numpy()
        out = []
        for b in range(self.n_inst):
            N = int(self.dims[b])
            base = self.n_store * self.off[b]
            out.append(h[base: base + self.n_store * N * N].reshape(self.n_store, N, N))
        return out
