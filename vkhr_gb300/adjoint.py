"""torch.autograd wrappers of the differentiable path (the check harness).

`raymarch(density, tangent, kd_exp, params, ctx, K)` renders through
vkhr_raymarch_train and differentiates through vkhr_raymarch_adjoint;
`splat(vertices, bounds, res, ctx)` is vkhr_splat_vertices with
vkhr_splat_vertices_adjoint as its backward.  Both call the C ABI on the
tensors' device memory; there is no other implementation behind them.
"""
import torch

from . import _abi


def _params_with(params, kd, exponent, exponent2=None):
    p = _abi.RaymarchParams.from_buffer_copy(params)
    p.kd = float(kd)
    p.hair_exponent = float(exponent)
    if exponent2 is not None:
        p.spec_exponent2 = float(exponent2)
    p.density_format = _abi.DENSITY_F32
    p.tangent_format = _abi.TANGENT_F32X4
    return p


class RaymarchFunction(torch.autograd.Function):
    """rgba (H, W, 4) = raymarch(density (n,), tangent (n, 4), kd_exp), kd_exp
    = (kd, hair_exponent) or (kd, hair_exponent, spec_exponent2)."""

    @staticmethod
    def forward(fctx, density, tangent, kd_exp, params, native, K):
        p = _params_with(params, *(float(x) for x in kd_exp.detach().cpu()))
        density = density.contiguous()
        tangent = tangent.contiguous()
        dev = density.device
        rgba = torch.empty((p.height, p.width, 4), dtype=torch.float32, device=dev)
        nbytes = native.tape_bytes(p, K)
        tape = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        s = torch.cuda.current_stream(dev).cuda_stream
        native.raymarch_train(p, density.data_ptr(), tangent.data_ptr(), rgba.data_ptr(), None, tape.data_ptr(),
                              nbytes, K, s)
        fctx.save_for_backward(density, tangent, tape)
        fctx.params, fctx.native, fctx.K, fctx.nparams = p, native, K, kd_exp.numel()
        return rgba

    @staticmethod
    def backward(fctx, g_rgba):
        density, tangent, tape = fctx.saved_tensors
        g_rgba = g_rgba.contiguous().float()
        gd = torch.zeros_like(density)
        gt = torch.zeros_like(tangent)
        gp = torch.zeros(3, dtype=torch.float64, device=density.device)  # kd, exponent, exponent2
        s = torch.cuda.current_stream(density.device).cuda_stream
        fctx.native.raymarch_adjoint(fctx.params, density.data_ptr(), tangent.data_ptr(), tape.data_ptr(), fctx.K,
                                     g_rgba.data_ptr(), gd.data_ptr(), gt.data_ptr(), gp.data_ptr(), s)
        return gd, gt, gp[:fctx.nparams], None, None, None


class SplatFunction(torch.autograd.Function):
    """density (w*h*d,) = trilinear splat of vertices (V, 3)."""

    @staticmethod
    def forward(fctx, vertices, bounds, res, native):
        vertices = vertices.contiguous()
        w, h, d = res
        dens = torch.zeros(w * h * d, dtype=torch.float32, device=vertices.device)
        s = torch.cuda.current_stream(vertices.device).cuda_stream
        native.splat_vertices(vertices.data_ptr(), vertices.shape[0], bounds, res, dens.data_ptr(), s)
        fctx.save_for_backward(vertices)
        fctx.bounds, fctx.res, fctx.native = bounds, res, native
        return dens

    @staticmethod
    def backward(fctx, g_dens):
        (vertices,) = fctx.saved_tensors
        g_dens = g_dens.contiguous().float()
        gv = torch.empty_like(vertices)
        s = torch.cuda.current_stream(vertices.device).cuda_stream
        fctx.native.splat_vertices_adjoint(vertices.data_ptr(), vertices.shape[0], fctx.bounds, fctx.res,
                                           g_dens.data_ptr(), gv.data_ptr(), s)
        return gv, None, None, None


def raymarch(density, tangent, kd_exp, params, native, K=16):
    return RaymarchFunction.apply(density, tangent, kd_exp, params, native, K)


def splat(vertices, bounds, res, native):
    return SplatFunction.apply(vertices, bounds, res, native)
