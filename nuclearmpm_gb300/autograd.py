"""Differentiable MPM rollouts for PyTorch: a torch.autograd.Function over the hand-written
adjoint of the step (nclr_rollout_* in include/nclr_gpu.h).

    roll = Rollout(x0, res=64, steps=2000, checkpoint_every=50)      # jelly
    xT, vT = roll(x0, v0, E, nu)           # CUDA tensors in, CUDA tensors out
    loss = ((xT.mean(0) - target) ** 2).sum()
    loss.backward()                        # gradients of x0, v0, E, nu

The forward pass runs the GPU step kernels and keeps a checkpoint every `checkpoint_every`
steps; the backward pass recomputes each segment from its checkpoint and runs the adjoint
kernels back through it.  Only the jelly material is covered (the rollout has no plasticity).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import capi


def _dp(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class Rollout:
    """A differentiable `steps`-step rollout of `n` particles of one material (`model`: jelly
    by default, or snow or liquid with their plasticity; positions x0 only size and place the
    simulation; mass / volume default to 1, as Particle<dim> does)."""

    def __init__(self, x0, *, res: int = 64, steps: int = 100, checkpoint_every: int = 50,
                 dt: float = 1e-4, gravity: float = -100.0, mass=None, volume=None,
                 physics: int = capi.PHYSICS_REFERENCE, device: int = 0, sort_interval: int = 8,
                 stress_model: int = capi.STRESS_COROTATED, profile: bool = False,
                 model: int = 1):
        x = np.ascontiguousarray(torch.as_tensor(x0).detach().cpu().numpy(), dtype=np.float32)
        self.n, self.dim = x.shape
        self.steps = int(steps)
        m = None if mass is None else np.ascontiguousarray(mass, dtype=np.float32)
        vo = None if volume is None else np.ascontiguousarray(volume, dtype=np.float32)
        opt = capi.default_options(physics=physics, device=device, sort_interval=sort_interval,
                                   stress_model=stress_model, profile=int(profile))
        h = ctypes.c_void_p()
        L = capi.lib()
        st = L.nclr_rollout_create_model(ctypes.byref(h), self.dim, self.n, x.ctypes.data,
                                         None if m is None else m.ctypes.data,
                                         None if vo is None else vo.ctypes.data, int(model),
                                         int(res), float(dt), float(gravity), self.steps,
                                         int(checkpoint_every), ctypes.byref(opt))
        if st != 0:
            raise capi.NclrError(st, (L.nclr_rollout_error(None) or b"").decode())
        self._h = h
        self.device = torch.device("cuda", device)
        self.corrected = physics == capi.PHYSICS_CORRECTED

    def _check(self, st):
        if st != 0:
            msg = (capi.lib().nclr_rollout_error(self._h) or b"").decode()
            if st == capi.NCLR_ERR_OUT_OF_RANGE:
                raise capi.OutOfRange(st, msg)
            raise capi.NclrError(st, msg)

    def __call__(self, x0, v0, E, nu, F0=None, C0=None):
        return RolloutFunction.apply(self, x0, v0, E, nu, F0, C0)

    def profile(self) -> dict:
        """Per kernel phase (capi.PHASE_NAMES): (total device ms, launches) since the last
        reset, with profile=True: the forward kernels of the forward pass and of the
        backward's recomputation, and the reverse kernels of every backward step."""
        out = {}
        for i, name in enumerate(capi.PHASE_NAMES):
            ms, k = ctypes.c_double(), ctypes.c_int64()
            self._check(capi.lib().nclr_rollout_profile_get(self._h, i, ctypes.byref(ms),
                                                            ctypes.byref(k)))
            out[name] = (float(ms.value), int(k.value))
        return out

    def profile_reset(self) -> None:
        self._check(capi.lib().nclr_rollout_profile_reset(self._h))

    def timing(self) -> tuple[float, float]:
        f, b = ctypes.c_double(), ctypes.c_double()
        capi.lib().nclr_rollout_timing(self._h, ctypes.byref(f), ctypes.byref(b))
        return f.value, b.value

    def close(self):
        if getattr(self, "_h", None):
            capi.lib().nclr_rollout_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RolloutFunction(torch.autograd.Function):
    """(x0, v0, E, nu[, F0, C0]) -> (x_T, v_T); backward via the adjoint rollout.  E and nu are
    the scene's pair (numbers or 0-d tensors) or one value per particle (tensors of n values,
    nclr_rollout_forward_moduli), with gradients of the same shape."""

    @staticmethod
    def forward(ctx, roll: Rollout, x0, v0, E, nu, F0=None, C0=None):
        dev = roll.device
        n, d = roll.n, roll.dim
        f32 = dict(dtype=torch.float32, device=dev)
        x0c = x0.detach().to(**f32).contiguous()
        v0c = v0.detach().to(**f32).contiguous()
        if F0 is None:  # Particle<dim>'s F = diag<dim>(1): diag(1,1,0) in 3D (src/nclr_math.h:13-19)
            F0c = torch.eye(d, **f32).expand(n, d, d).contiguous()
            if d == 3 and not roll.corrected:
                F0c[:, 2, 2] = 0.0
        else:
            F0c = F0.detach().to(**f32).contiguous()
        C0c = torch.zeros(n, d, d, **f32) if C0 is None else C0.detach().to(**f32).contiguous()
        xT = torch.empty(n, d, **f32)
        vT = torch.empty(n, d, **f32)
        per_particle = torch.is_tensor(E) and E.numel() > 1
        if per_particle:
            Ec = E.detach().to(**f32).reshape(n).contiguous()
            nuc = torch.as_tensor(nu).detach().to(**f32).reshape(n).contiguous()
            ctx.moduli = (Ec, nuc)  # kept alive until the call below has read them
            ctx.shapes = (E.shape, torch.as_tensor(nu).shape)
            torch.cuda.synchronize(dev)
            roll._check(capi.lib().nclr_rollout_forward_moduli(
                roll._h, _dp(x0c), _dp(v0c), _dp(F0c), _dp(C0c), _dp(Ec), _dp(nuc), _dp(xT),
                _dp(vT), None, None))
        else:
            Ef, nuf = float(E), float(nu)
            torch.cuda.synchronize(dev)
            roll._check(capi.lib().nclr_rollout_forward(roll._h, _dp(x0c), _dp(v0c), _dp(F0c),
                                                         _dp(C0c), Ef, nuf, _dp(xT), _dp(vT),
                                                         None, None))
        ctx.per_particle = per_particle
        ctx.roll = roll
        ctx.params = [(t.dtype, t.device) if torch.is_tensor(t) else None for t in (E, nu)]
        ctx.given = (F0 is not None, C0 is not None)
        return xT, vT

    @staticmethod
    def backward(ctx, gxT, gvT):
        roll = ctx.roll
        dev = roll.device
        n, d = roll.n, roll.dim
        f32 = dict(dtype=torch.float32, device=dev)
        gx = None if gxT is None else gxT.to(**f32).contiguous()
        gv = None if gvT is None else gvT.to(**f32).contiguous()
        gx0 = torch.empty(n, d, **f32)
        gv0 = torch.empty(n, d, **f32)
        gF0 = torch.empty(n, d, d, **f32)
        gC0 = torch.empty(n, d, d, **f32)
        torch.cuda.synchronize(dev)
        out = []
        if ctx.per_particle:
            gEp = torch.empty(n, **f32)
            gnup = torch.empty(n, **f32)
            roll._check(capi.lib().nclr_rollout_backward_moduli(
                roll._h, _dp(gx), _dp(gv), None, None, _dp(gx0), _dp(gv0), _dp(gF0), _dp(gC0),
                _dp(gEp), _dp(gnup)))
            for val, spec, shape in ((gEp, ctx.params[0], ctx.shapes[0]),
                                     (gnup, ctx.params[1], ctx.shapes[1])):
                out.append(None if spec is None
                           else val.to(dtype=spec[0], device=spec[1]).reshape(shape))
        else:
            gE, gnu = ctypes.c_double(), ctypes.c_double()
            roll._check(capi.lib().nclr_rollout_backward(roll._h, _dp(gx), _dp(gv), None, None,
                                                          _dp(gx0), _dp(gv0), _dp(gF0), _dp(gC0),
                                                          ctypes.byref(gE), ctypes.byref(gnu)))
            for val, spec in ((gE.value, ctx.params[0]), (gnu.value, ctx.params[1])):
                out.append(None if spec is None else torch.tensor(val, dtype=spec[0], device=spec[1]))
        return (None, gx0, gv0, out[0], out[1], gF0 if ctx.given[0] else None,
                gC0 if ctx.given[1] else None)
