"""FWI through torch autograd.

The reference builds its FWI objective from two operators:
``NonLinearOperator(wemOp, bornOp)`` inside python-solver's
``ProblemL2NonLinear`` (scripts/fwi.py:70-71,90,113).  The objective is
``1/2 ||WEM(m) - d_obs||^2``, and its gradient is the Born adjoint of the
residual at the current background (BornFull::adjoint,
propagator/src/born_prop.cpp:178-216).

``FWIGradient`` is that pair as a ``torch.autograd.Function``:
- forward: the nonlinear modelling of ``WemOp``;
- backward: ``BornOp.adjoint`` of the incoming data gradient, with the
  background set to the forward's model.

Both run on the CUDA library.  For any loss of the synthetic data, the
leaves get the reference's Born-linearised gradient:
- compat adjoint (default): the reference as coded;
- exact adjoint: the transpose of the Born operator.

For a real loss and complex leaves, torch's gradient is dL/dRe + i dL/dIm.
That is B^H r for real time data r, which is what the Born adjoint returns.

``WEMGradient`` is the same forward with the exact derivative as its
backward: the adjoint-state gradient of the modelled data itself (through
Reflect, the split step, the phase shift and the reference slowness; the
library's ``wem_gradient``), which a finite-difference check of the
modelling pins.  Its ``checkpoint`` k > 1 keeps every k-th depth's
wavefields and recomputes the depths between (same numbers, bit for bit).

Memory: the Born adjoint stores two or three wavefields per (shot,
frequency) row, the exact gradient four (or two every k depths with
checkpointing).  The library also bounds the storage by running the rows
in chunks sized to free HBM.
"""
from __future__ import annotations

import numpy as np
import torch

from .core import BornOp, FwiOp, WemOp
from .params import WemParams


class FWIGradient(torch.autograd.Function):
    """d = WEM(s2, rho); backward: (g_s2, g_rho) = Born^H(dL/dd) at (s2, rho)."""

    @staticmethod
    def forward(ctx, s2, rho, wem: WemOp, born: BornOp):
        if not (s2.is_cuda and rho.is_cuda):
            raise ValueError("FWIGradient works on CUDA tensors")
        s2c, rhoc = s2.detach().contiguous(), rho.detach().contiguous()
        d = torch.empty(wem.data_shape(0), dtype=torch.float32, device=s2.device)
        wem.forward(s2c, rhoc, d)
        ctx.save_for_backward(s2c, rhoc)
        ctx.born = born
        return d

    @staticmethod
    def backward(ctx, grad_d):
        s2, rho = ctx.saved_tensors
        born: BornOp = ctx.born
        born.set_background(s2, rho)
        g_s2, g_rho = torch.zeros_like(s2), torch.zeros_like(rho)
        born.adjoint(g_s2, g_rho, grad_d.contiguous())
        return g_s2, g_rho, None, None


class WEMGradient(torch.autograd.Function):
    """d = WEM(s2, rho); backward: (g_s2, g_rho) = J^H(dL/dd), J the exact
    derivative of the modelling at (s2, rho)."""

    @staticmethod
    def forward(ctx, s2, rho, wem: WemOp, checkpoint: int = 0):
        if not (s2.is_cuda and rho.is_cuda):
            raise ValueError("WEMGradient works on CUDA tensors")
        s2c, rhoc = s2.detach().contiguous(), rho.detach().contiguous()
        d = torch.empty(wem.data_shape(0), dtype=torch.float32, device=s2.device)
        wem.forward(s2c, rhoc, d)
        ctx.save_for_backward(s2c, rhoc)
        ctx.wem, ctx.checkpoint = wem, int(checkpoint)
        return d

    @staticmethod
    def backward(ctx, grad_d):
        s2, rho = ctx.saved_tensors
        g_s2, g_rho = torch.zeros_like(s2), torch.zeros_like(rho)
        ctx.wem.gradient(s2, rho, grad_d.contiguous(), g_s2, g_rho, checkpoint=ctx.checkpoint)
        return g_s2, g_rho, None, None


def modelled_data(s2, rho, wem: WemOp, born: BornOp = None, exact: bool = False, checkpoint: int = 0):
    """Synthetic data of (s2, rho) that backpropagates through the Born
    adjoint (the reference's gradient) or, with exact=True, through the
    exact derivative of the modelling."""
    if exact:
        return WEMGradient.apply(s2, rho, wem, checkpoint)
    return FWIGradient.apply(s2, rho, wem, born)


class Reflectivity3D(torch.autograd.Function):
    """d = L r with L the 3D reflectivity Born (``Refl3DOp``; BornRefl's
    operator on planes); backward: the migration L^H(dL/dd).  The forward's
    stored background field is kept every ``checkpoint`` depths (k > 1) and
    recomputed between, with the same numbers."""

    @staticmethod
    def forward(ctx, model, op, checkpoint: int = 0):
        if not model.is_cuda:
            raise ValueError("Reflectivity3D works on CUDA tensors")
        d = torch.empty(op.data_shape(0), dtype=torch.float32, device=model.device)
        op.forward(model.detach().contiguous(), d, checkpoint=int(checkpoint))
        ctx.op = op
        return d

    @staticmethod
    def backward(ctx, grad_d):
        op = ctx.op
        img = torch.zeros(op.model_shape, dtype=torch.complex64, device=grad_d.device)
        op.adjoint(img, grad_d.contiguous())
        return img, None, None


def reflectivity_data_3d(model, op, checkpoint: int = 0):
    """Synthetic data of a 3D reflectivity that backpropagates through the
    migration (least-squares migration gradients)."""
    return Reflectivity3D.apply(model, op, checkpoint)


class FwiObjective:
    """The L2 FWI objective and its gradient, one call per iteration.

    ``obj(s2, rho) -> (loss, g_s2, g_rho)``, with
    loss = 1/2 ||WEM(s2, rho) - d_obs||^2 and g = Born^H(WEM(s2, rho) - d_obs),
    computed by one library call (``FwiOp``, ``fwi_gradient``): the residual
    and loss stay on the device and the background tables are built once.

    d_obs (``[ns][nr][nt]`` float32, numpy or a CUDA tensor) is copied to the
    device once.  Models may be numpy arrays (the call copies them in, and the
    gradients out, through pinned buffers) or CUDA tensors (no copies; the
    gradients are returned as new CUDA tensors).
    """

    def __init__(self, p: WemParams, wavelet, d_obs, device=None, exact=False, checkpoint=0):
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.exact, self.checkpoint = bool(exact), int(checkpoint)
        self.op = FwiOp(p, wavelet)
        self.d_obs = torch.as_tensor(d_obs).to(self.device, torch.float32).contiguous()
        if tuple(self.d_obs.shape) != tuple(self.op.data_shape(0)):
            raise ValueError(f"d_obs shape {tuple(self.d_obs.shape)} != {self.op.data_shape(0)}")
        shape = self.op.model_shape
        self._dev_in = [torch.empty(shape, dtype=torch.complex64, device=self.device) for _ in range(2)]
        self._pin_out = [torch.empty(shape, dtype=torch.complex64).pin_memory() for _ in range(2)]
        self.h2d_bytes = 0
        self.d2h_bytes = 0

    def _to_device(self, a, i):
        if isinstance(a, torch.Tensor) and a.is_cuda:
            return a.contiguous(), False
        t = torch.as_tensor(np.ascontiguousarray(a, dtype=np.complex64))
        self._dev_in[i].copy_(t, non_blocking=t.is_pinned())
        self.h2d_bytes = t.numel() * 8 * 2
        return self._dev_in[i], True

    def __call__(self, s2, rho):
        s2_d, host = self._to_device(s2, 0)
        rho_d, _ = self._to_device(rho, 1)
        g0 = torch.empty_like(s2_d)
        g1 = torch.empty_like(rho_d)
        loss = self.op.gradient(s2_d, rho_d, self.d_obs, g0, g1, exact=self.exact, checkpoint=self.checkpoint)
        if not host:
            return loss, g0, g1
        self._pin_out[0].copy_(g0)
        self._pin_out[1].copy_(g1)
        self.d2h_bytes = 2 * g0.numel() * 8 + 8
        return loss, self._pin_out[0].numpy().copy(), self._pin_out[1].numpy().copy()
