"""torch.autograd bindings of the EM-ICP and Softassign adjoints
(cesa_emicp_forward_device / cesa_emicp_backward_device and
cesa_softassign_forward_device / cesa_softassign_backward_device), for
gradient checks.

    R, t = emicp_autograd(X, Y, R0, t0, param)
    R, t = softassign_autograd(X, Y, R0, t0, param)

X (N, 3), Y (M, 3), R0 (3, 3), t0 (3) are float32 CUDA tensors; R, t are the
registered pose. backward() returns dL/dX, dL/dY, dL/dR0 and dL/dt0; use
se3_gradient() for the gradient with respect to a perturbation
(exp(w) R0, t0 + v) of the initial pose.
"""
import ctypes

import torch

from . import Params, _check, _dptr, _stream_handle, lib


def _soa(P):
    return P.detach().to(torch.float32).t().contiguous().reshape(-1)


class _TapedFunction(torch.autograd.Function):
    """Forward records a tape on the device; backward replays it in reverse."""
    _name = None

    @classmethod
    def _fns(cls, L):
        return (getattr(L, "cesa_%s_tape_bytes" % cls._name), getattr(L, "cesa_%s_forward_device" % cls._name),
                getattr(L, "cesa_%s_backward_device" % cls._name))

    @classmethod
    def forward(cls, ctx, X, Y, R0, t0, param):
        L = lib()
        tape_bytes, fwd, _ = cls._fns(L)
        N, M = X.shape[0], Y.shape[0]
        dX, dY = _soa(X), _soa(Y)
        rt = torch.cat([R0.detach().reshape(-1), t0.detach().reshape(-1)]).to(torch.float32).contiguous()
        nbytes = tape_bytes(N, M, ctypes.byref(param))
        if nbytes == 0:
            raise ValueError("invalid %s arguments" % cls._name)
        tape = torch.empty(nbytes, dtype=torch.uint8, device=X.device)
        stream = ctypes.c_void_p(_stream_handle(None))
        _check(fwd(_dptr(dX), N, _dptr(dY), M, _dptr(rt), ctypes.byref(param), _dptr(tape), None, stream),
               "%s_forward_device" % cls._name)
        ctx.tape, ctx.param, ctx.N, ctx.M = tape, param, N, M
        return rt[:9].reshape(3, 3).clone(), rt[9:].clone()

    @classmethod
    def backward(cls, ctx, gR, gt):
        L = lib()
        _, _, bwd = cls._fns(L)
        N, M = ctx.N, ctx.M
        dev = ctx.tape.device
        g = torch.cat([(gR if gR is not None else torch.zeros(3, 3, device=dev)).reshape(-1),
                       (gt if gt is not None else torch.zeros(3, device=dev)).reshape(-1)]).to(torch.float32)
        g = g.contiguous()
        gX = torch.empty(3 * N, dtype=torch.float32, device=dev)
        gY = torch.empty(3 * M, dtype=torch.float32, device=dev)
        g0 = torch.empty(12, dtype=torch.float32, device=dev)
        _check(bwd(N, M, ctypes.byref(ctx.param), _dptr(ctx.tape), _dptr(g), _dptr(gX), _dptr(gY), _dptr(g0), None,
                   ctypes.c_void_p(_stream_handle(None))), "%s_backward_device" % cls._name)
        return gX.reshape(3, N).t(), gY.reshape(3, M).t(), g0[:9].reshape(3, 3), g0[9:], None


class EmicpFunction(_TapedFunction):
    _name = "emicp"


class SoftassignFunction(_TapedFunction):
    _name = "softassign"


def softassign_autograd(X, Y, R0, t0, param=None):
    return SoftassignFunction.apply(X, Y, R0, t0, param or Params.default())


def emicp_autograd(X, Y, R0, t0, param=None):
    return EmicpFunction.apply(X, Y, R0, t0, param or Params.default())


def se3_gradient(R0, gR0, gt0):
    """(dL/dw, dL/dv) for the initial pose exp(w) R0, t0 + v at w = v = 0:
    dL/dw = vee(G - G^T) with G = dL/dR0 R0^T, dL/dv = dL/dt0."""
    G = gR0 @ R0.t()
    gw = torch.stack([G[2, 1] - G[1, 2], G[0, 2] - G[2, 0], G[1, 0] - G[0, 1]])
    return gw, gt0
