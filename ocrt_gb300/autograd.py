"""torch.autograd face of the adjoint solve (ocrt_gb_solve_batch_adjoint).

PyTorch is only the carrier of tensors and the autograd graph here; every
solve and every derivative is computed by the CUDA library.

    rho = sos_reflectance(dtau, ssa, wind, cases, opts, aerosols)

dtau, ssa: [n, nt] layer optical depths and single-scattering albedos (layer
l spans levels l..l+1, TOA first); wind: [n] wind speeds in m/s.  rho: [n, 3]
= (rho_I, rho_Q, rho_U) at each case's view geometry.  When any input needs a
gradient, the forward call also returns the full 3-row Jacobian of every pixel
from the library's adjoint sweep (three cotangent rows in the same device
pass), and backward contracts it with the incoming gradient.
"""
import copy

import numpy as np
import torch

from . import _abi
from . import layer_defaults, solve_batch_adjoint


class SOSReflectance(torch.autograd.Function):
    @staticmethod
    def forward(ctx, dtau, ssa, wind, cases, opts, aerosols):
        if dtau.dim() != 2 or ssa.shape != dtau.shape or wind.shape != (dtau.shape[0],):
            raise ValueError("dtau, ssa must be [n, nt] and wind [n]")
        n, nt = dtau.shape
        if len(cases) != n:
            raise ValueError("one case per row of dtau")
        dt = dtau.detach().to("cpu", torch.float64).numpy()
        ss = ssa.detach().to("cpu", torch.float64).numpy()
        ww = wind.detach().to("cpu", torch.float64).numpy()
        cs = []
        for i in range(n):
            c = copy.copy(cases[i])
            c.wind_speed = float(ww[i])
            cs.append(c)
        layers = [_abi.LayersHolder(nt, dt[i], ss[i]) for i in range(n)]
        need = any(ctx.needs_input_grad[:3])
        cot = np.broadcast_to(np.eye(3), (n, 3, 3)).copy() if need else None
        res, g = solve_batch_adjoint(cs, opts, aerosols, layers, cot)
        rho = np.stack([res["rho_I"], res["rho_Q"], res["rho_U"]], axis=1)
        out = torch.as_tensor(rho, dtype=dtau.dtype, device=dtau.device)
        if need:
            to = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=dtau.dtype, device=dtau.device)
            ctx.save_for_backward(to(g["d_dtau"][:, :, :nt]), to(g["d_ssa"][:, :, :nt]), to(g["d_wind"]))
        return out

    @staticmethod
    def backward(ctx, grad_rho):
        jt, js, jw = ctx.saved_tensors                  # [n, 3, nt], [n, 3, nt], [n, 3]
        gd = torch.einsum("nr,nrl->nl", grad_rho, jt) if ctx.needs_input_grad[0] else None
        gs = torch.einsum("nr,nrl->nl", grad_rho, js) if ctx.needs_input_grad[1] else None
        gw = (grad_rho * jw).sum(dim=1) if ctx.needs_input_grad[2] else None
        return gd, gs, gw, None, None, None


def sos_reflectance(dtau, ssa, wind, cases, opts, aerosols=None):
    """Differentiable TOA reflectance (see the module docstring)."""
    return SOSReflectance.apply(dtau, ssa, wind, cases, opts, aerosols)


def layer_parameters(cases, opts, aerosols=None, dtype=torch.float64):
    """Profile values of (dtau [n, nt], ssa [n, nt], wind [n]) to start from."""
    n = len(cases)
    ol = opts if isinstance(opts, (list, tuple)) else [opts] * n
    al = aerosols if isinstance(aerosols, (list, tuple)) else [aerosols] * n
    pairs = [layer_defaults(cases[i], ol[i], al[i]) for i in range(n)]
    dt = torch.tensor(np.stack([p[0] for p in pairs]), dtype=dtype)
    ss = torch.tensor(np.stack([p[1] for p in pairs]), dtype=dtype)
    w = torch.tensor([c.wind_speed for c in cases], dtype=dtype)
    return dt, ss, w
