"""Learned initial guess for the pressure-correction (p') equation.

Host side of the network in csrc/lp.cu: parameters, training steps and
inference through the C ABI, with device buffers held as torch tensors
(torch is used only for device memory here; every kernel is the library's).

  lp = LearnedPressure((nx, ny, nz), seed=1)      # buffers for grids up to nx*ny*nz voxels
  samples = collect_samples([configs.small_furnace()], iters=40, every=4, nsweeps=40)
  lp.fit(samples, steps=300, lr=1e-3)
  solver.set_lp(lp)                               # p' solves start from the network's guess
"""
from __future__ import annotations

import ctypes as C
import random

import numpy as np

from . import abi
from .solver import Case, GfmError, GpuSolver


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise GfmError(abi.GFM_E_NODEVICE, "no CUDA device: the learned preconditioner has no CPU path")
    return torch


class LearnedPressure:
    """3-D convolutional encoder-decoder, BF16 tensor-core kernels, FP32 master weights and Adam."""

    def __init__(self, dims: tuple, seed: int = 1, lib: C.CDLL | None = None):
        self.lib = lib or abi.load_library()
        self.dims = tuple(int(d) for d in dims)
        h = C.c_void_p()
        rc = self.lib.gfm_lp_create(*self.dims, seed, C.byref(h))
        if rc != abi.GFM_OK:
            raise GfmError(rc, self.lib.gfm_lp_last_error().decode())
        self.h = h
        self.n = self.lib.gfm_lp_num_params()

    def params(self) -> np.ndarray:
        p = np.zeros(self.n, np.float32)
        self._check(self.lib.gfm_lp_get_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float)), None))
        return p

    def grads(self) -> np.ndarray:
        g = np.zeros(self.n, np.float32)
        self._check(self.lib.gfm_lp_get_params(self.h, None, g.ctypes.data_as(C.POINTER(C.c_float))))
        return g

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n
        self._check(self.lib.gfm_lp_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))))

    def set_tensor_path(self, tcgen05: bool) -> None:
        """Forward convolutions on tcgen05 (True) or mma.sync (False)."""
        self._check(self.lib.gfm_lp_set_tensor_path(self.h, 1 if tcgen05 else 0))

    def tensor_status(self) -> int:
        """0: every tcgen05 tile's first bounded wait for its MMAs succeeded;
        1: a first wait ran out and the second saw the MMAs end (output
        written); 2: a tile gave up (the forward pass's output invalid)."""
        return self.lib.gfm_lp_tensor_status(self.h)

    def forward(self, feats, dims) -> "torch.Tensor":
        torch = _torch()
        out = torch.empty(int(np.prod(dims)), dtype=torch.float32, device=feats.device)
        self._check(self.lib.gfm_lp_forward(self.h, feats.data_ptr(), out.data_ptr(), *dims, None))
        torch.cuda.synchronize()
        return out

    def train_step(self, feats, target, dims, lr: float = 1e-3, update: bool = True) -> float:
        loss = C.c_double()
        self._check(self.lib.gfm_lp_train_step(self.h, feats.data_ptr(), target.data_ptr(), *dims, lr,
                                               1 if update else 0, C.byref(loss), None))
        return loss.value

    def fit(self, samples: list, steps: int, lr: float = 1e-3, seed: int = 0) -> list:
        """Adam over randomly drawn samples; returns the loss of every step."""
        rnd = random.Random(seed)
        hist = []
        for _ in range(steps):
            f, t, d = samples[rnd.randrange(len(samples))]
            hist.append(self.train_step(f, t, d, lr))
        return hist

    def _check(self, rc: int) -> None:
        if rc != abi.GFM_OK:
            raise GfmError(rc, self.lib.gfm_lp_last_error().decode())

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.gfm_lp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pcorr_sample(solver: GpuSolver, nsweeps: int):
    """(inputs, target, dims) of the p' system of the solver's last iteration;
    the target is its solution after `nsweeps` line-solver sweeps from zero,
    scaled to unit RMS over the open cells."""
    torch = _torch()
    g = solver.case
    dims = (g.mp // 2 - 2, g.np // 2 - 2, g.lp // 2 - 2)
    nv = int(np.prod(dims))
    feats = torch.empty((nv, 16), dtype=torch.bfloat16, device="cuda")
    tgt = torch.empty(nv, dtype=torch.float32, device="cuda")
    d = (C.c_int * 3)()
    solver._check(solver.lib.gfm_gpu_pcorr_sample(solver.h, nsweeps, feats.data_ptr(), tgt.data_ptr(), d))
    assert tuple(d) == dims
    return feats, tgt, dims


def train_default(dims: tuple, seed: int = 3, variants: int = 8, log: list | None = None,
                  steps: int = 1500) -> LearnedPressure:
    """The standard recipe: p' systems of `variants` seeded variants of the
    48x24x16 furnace (one every 5 outer iterations from 5 to 120, targets from
    60 sweeps), `steps` Adam steps at 2e-3 and as many at 5e-4.  `dims` sizes
    the network's buffers for the largest grid it will be applied to."""
    from . import configs
    samples = collect_samples([configs.furnace_variant(s) for s in range(variants)], iters=120, every=5, nsweeps=60,
                              start=5)
    lp = LearnedPressure(dims, seed=seed)
    for lr in (2e-3, 5e-4):
        h = lp.fit(samples, steps=steps, lr=lr, seed=seed)
        if log is not None:
            log.append({"lr": lr, "steps": steps, "loss_first": float(np.mean(h[:50])), "loss_last": float(np.mean(h[-50:]))})
    return lp


def collect_samples(cfgs: list, iters: int, every: int, nsweeps: int, precision: int = abi.GFM_PREC_MIXED,
                    start: int = 1) -> list:
    """Samples from the plain solver: for each case, one every `every` outer
    iterations from iteration `start` up to `iters`."""
    out = []
    for cfg in cfgs:
        case = Case(cfg)
        s = GpuSolver(case, adi_mode=abi.GFM_ADI_REDBLACK, precision=precision)
        s.start()
        done = 0
        if start > 1:
            s.gflow(start - 1)
            done = start - 1
        while done < iters:
            s.gflow(1)
            done += 1
            if (done - start) % every == 0:
                out.append(pcorr_sample(s, nsweeps))
        s.close()
    return out
