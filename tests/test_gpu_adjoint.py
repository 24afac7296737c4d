"""The differentiable path on the GPU: the training forward equals
vkhr_raymarch bit for bit; the adjoint (vkhr_raymarch_adjoint) against FP64
central finite differences (h = 1e-3) of the FP64 oracle's loss on 256
random coordinates (densities of nonzero voxels, tangent components) and on
kd and both specular exponents (ill-conditioned coordinates excluded as in
tests/test_oracle_adjoint.py), and against the oracle's FP64 analytic
gradient on every coordinate; for the reference's shading, the workloads'
dual-lobe Kajiya-Kay and the directional AO; the result does not depend on
the checkpoint interval; the splat and its adjoint against the FP64 oracle,
and the chained vertex gradient through torch.autograd (the check harness)."""
import numpy as np
import pytest

from vkhr_gb300 import _abi, adjoint, scene
from tests.test_oracle_adjoint import FLOOR, H, SHADINGS, TOL, central, diff_scene

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def _shading_params(p):
    """kd and the exponents the gradient is taken with respect to."""
    return [p.kd, p.hair_exponent] + ([p.spec_exponent2] if p.spec_exponent2 > 0 else [])


def _fd_params(O, p, dens, tan, target, mask=None):
    """FP64 central differences (h = 1e-3 relative to 1, over the stored
    float32 values) of the oracle's loss with respect to kd and the
    exponents, with the h / 2 agreement check; None where ill-conditioned."""
    out = []
    for field in ("kd", "hair_exponent", "spec_exponent2")[:len(_shading_params(p))]:
        fds = []
        for h in (H, H / 2):
            qs = []
            for x in (getattr(p, field) - h, getattr(p, field) + h):
                q = _abi.RaymarchParams.from_buffer_copy(p)
                setattr(q, field, x)
                qs.append(q)
            lo, hi = (O.diff_loss(q, dens, tan, target, mask=mask) for q in qs)
            fds.append((hi - lo) / (getattr(qs[1], field) - getattr(qs[0], field)))
        ok = abs(fds[0] - fds[1]) <= max(TOL * max(abs(fds[0]), abs(fds[1])), FLOOR)
        out.append(fds[0] if ok else None)
    return out


def _gpu_grads(ctx, torch, p, dens, tan, target, K, mask=None):
    """GPU loss gradient: (loss, g_density, g_tangent, g_params, rgba); the
    loss runs over the pixels where mask (H, W) is true (None: all)."""
    d = _dev(torch, dens).requires_grad_(True)
    t = _dev(torch, tan).requires_grad_(True)
    kp = torch.tensor(_shading_params(p), dtype=torch.float64, device="cuda", requires_grad=True)
    rgba = adjoint.raymarch(d, t, kp, p, ctx, K)
    sq = (rgba.double() - _dev(torch, target).double()) ** 2
    if mask is not None:
        sq = sq * torch.from_numpy(mask.astype(np.float64)).cuda()[..., None]
    loss = sq.sum()
    loss.backward()
    torch.cuda.synchronize()
    return (float(loss.detach()), d.grad.double().cpu().numpy(), t.grad.double().cpu().numpy(), kp.grad.cpu().numpy(),
            rgba.detach().cpu().numpy())


@pytest.mark.parametrize("steps", [64.0, 100.0])
def test_train_forward_equals_raymarch(ctx, oracle_lib, steps):
    import torch

    st, b, p, dens, tan, target = diff_scene(oracle_lib, size=(96, 72), steps=steps)
    d, t = _dev(torch, dens), _dev(torch, tan)
    ref = torch.empty((p.height, p.width, 4), dtype=torch.float32, device="cuda")
    ctx.raymarch(p, d.data_ptr(), t.data_ptr(), None, ref.data_ptr(), None)
    for K in (7, 16):
        out = torch.empty_like(ref)
        nbytes = ctx.tape_bytes(p, K)
        tape = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        ctx.raymarch_train(p, d.data_ptr(), t.data_ptr(), out.data_ptr(), None, tape.data_ptr(), nbytes, K)
        torch.cuda.synchronize()
        assert torch.equal(out, ref)
    assert (ref[..., 3] > 0).sum().item() > 100


@pytest.mark.parametrize("shading,steps", [("reference", 64.0), ("reference", 100.0), ("dual_lobe", 64.0),
                                           ("dual_lobe_ao16", 100.0)])
def test_adjoint_vs_finite_differences(ctx, oracle_lib, shading, steps):
    """256 coordinates: 200 densities of nonzero voxels, 54 tangent components,
    kd and the exponents (2 or 3)."""
    import torch

    O = oracle_lib
    st, b, p, dens, tan, target = diff_scene(O, steps=steps, shading=SHADINGS[shading])
    d32, t32 = dens.astype(np.float32).astype(np.float64), tan.astype(np.float32).astype(np.float64)
    loss, gd, gt, gp, rgba = _gpu_grads(ctx, torch, p, d32, t32, target, 16)
    rng = np.random.default_rng(11)
    dcoords = rng.choice(np.nonzero((gd != 0) & (d32 > 0))[0], size=200, replace=False)
    tt = np.nonzero(np.abs(gt[:, :3]).sum(axis=1))[0]
    tcoords = list(zip(rng.choice(tt, size=54, replace=False).tolist(), rng.integers(0, 3, 54).tolist()))

    def fd(kind, c, h):
        if kind == "d":
            def f(x):
                dd = d32.copy()
                dd[c] = x
                return O.diff_loss(p, dd, t32, target)
            return central(f, d32[c], h)
        v, k = c
        def f(x):
            tt2 = t32.copy()
            tt2[v, k] = x
            return O.diff_loss(p, d32, tt2, target)
        return central(f, t32[v, k], h)

    got, want, ill, n = [], [], 0, 0
    for kind, coords, g in (("d", dcoords, lambda c: gd[c]), ("t", tcoords, lambda c: gt[c[0], c[1]])):
        for c in coords:
            n += 1
            (f1, dev1), (f2, dev2) = fd(kind, c, H), fd(kind, c, H / 2)
            if (dev1 > 1e-13 and dev2 > 0.5 * dev1) or abs(f1 - f2) > max(TOL * max(abs(f1), abs(f2)), FLOOR):
                ill += 1
                continue
            got.append(g(c))
            want.append(f1)
    assert n == 254 and ill <= 0.1 * n, ill
    got, want = np.array(got), np.array(want)
    # 1e-3 relative, normwise over the coordinates: the FP32 forward's image
    # (which dL/drgba is formed from) differs from the FP64 one by ~1e-5
    rel = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert rel <= TOL, rel
    # each coordinate within 1e-2, but for a few whose pixels take another
    # discrete decision (surface point) in FP32 than in FP64
    far = np.abs(got - want) > np.maximum(1e-2 * np.abs(want), FLOOR)
    assert far.sum() <= 0.02 * n, (far.sum(), got[far][:4], want[far][:4])
    # kd and the exponents against their own central differences (1e-3
    # relative) and against the oracle's analytic value
    fdp = _fd_params(O, p, d32, t32, target)
    assert sum(f is None for f in fdp) == 0, fdp
    for k, f in enumerate(fdp):
        assert abs(gp[k] - f) <= max(TOL * abs(f), FLOOR), (k, gp[k], f)
    _, _, _, gp_ref = O.diff_loss(p, d32, t32, target, grads=True)
    assert np.allclose(gp, gp_ref[:len(gp)], rtol=1e-3, atol=FLOOR), (gp, gp_ref)


@pytest.mark.parametrize("shading", sorted(SHADINGS))
def test_adjoint_vs_oracle_gradient(ctx, oracle_lib, shading):
    """Every coordinate against the oracle's FP64 analytic gradient (relative L2)."""
    import torch

    O = oracle_lib
    st, b, p, dens, tan, target = diff_scene(O, res=(40, 40, 40), size=(128, 96), steps=128.0, seed=6,
                                             shading=SHADINGS[shading])
    d32, t32 = dens.astype(np.float32).astype(np.float64), tan.astype(np.float32).astype(np.float64)
    loss, gd, gt, gp, rgba = _gpu_grads(ctx, torch, p, d32, t32, target, 32)
    lref, gd_ref, gt_ref, gp_ref = O.diff_loss(p, d32, t32, target, grads=True)
    assert abs(loss - lref) <= 1e-4 * lref
    for g, r in ((gd, gd_ref), (gt[:, :3], gt_ref[:, :3])):
        assert np.linalg.norm(g - r) <= 1e-3 * np.linalg.norm(r), np.linalg.norm(g - r) / np.linalg.norm(r)
    # kd and the exponents are sums over 12,288 pixels of terms of both signs;
    # the cancellation amplifies the FP32 image's error (dL/drgba is formed
    # from it): measured up to 7e-4 of the net sum (kd, reference shading)
    print("shading params", shading, gp, gp_ref[:len(gp)])
    assert np.allclose(gp, gp_ref[:len(gp)], rtol=1e-3), (gp, gp_ref)


def test_checkpoint_interval_does_not_matter(ctx, oracle_lib):
    import torch

    st, b, p, dens, tan, target = diff_scene(oracle_lib, size=(96, 72), steps=128.0)
    res = [_gpu_grads(ctx, torch, p, dens, tan, target, K) for K in (16, 32, 64)]
    for r in res[1:]:
        assert r[0] == res[0][0]
        assert np.linalg.norm(r[1] - res[0][1]) <= 1e-5 * np.linalg.norm(res[0][1])
        assert np.linalg.norm(r[2] - res[0][2]) <= 1e-5 * np.linalg.norm(res[0][2])


def test_splat_and_vertex_gradient(ctx, oracle_lib):
    """splat(V) on the GPU against the FP64 oracle; dL/dV of the loss of
    raymarch(splat(V)) through torch.autograd against the oracle's chain
    (FP64 loss gradient -> FP64 splat adjoint), and, on the 24 vertex
    coordinates of largest gradient, against FP64 central differences of the
    oracle's loss of raymarch(splat(V)) (h = 1e-3 and h / 2 must agree,
    else the coordinate is excluded; relative L2 <= 1e-3 over the rest)."""
    import torch

    O = oracle_lib
    st, b, p, dens, tan, target = diff_scene(O, size=(96, 72), steps=64.0)
    res = tuple(p.volume_resolution)
    V = torch.from_numpy(st.vertices).cuda().requires_grad_(True)
    dg = adjoint.splat(V, b, res, ctx)
    d_ref = O.splat(st.vertices, b, res)
    assert np.abs(dg.detach().double().cpu().numpy() - d_ref).max() <= 1e-4 * max(1.0, d_ref.max())
    t = _dev(torch, tan)
    kp = torch.tensor(_shading_params(p), dtype=torch.float64, device="cuda")
    rgba = adjoint.raymarch(dg, t, kp, p, ctx, 16)
    loss = ((rgba.double() - _dev(torch, target).double()) ** 2).sum()
    loss.backward()
    gv = V.grad.double().cpu().numpy()
    _, gd_ref, _, _ = O.diff_loss(p, dg.detach().double().cpu().numpy(), tan.astype(np.float32), target, grads=True)
    gv_ref = O.splat_adjoint(st.vertices, b, res, gd_ref)
    assert np.linalg.norm(gv_ref) > 0
    rel_chain = np.linalg.norm(gv - gv_ref) / np.linalg.norm(gv_ref)
    assert rel_chain <= 2e-4, rel_chain  # measured 1.4e-5

    # FP64 central differences of the oracle's loss with respect to vertex coordinates
    t32 = tan.astype(np.float32)

    def loss_at(v):
        return O.diff_loss(p, O.splat(v, b, res), t32, target)

    coords = np.argsort(-np.abs(gv_ref).ravel())[:24]
    got, want = [], []
    for c in coords:
        fds = []
        for h in (H, H / 2):
            lo_v, hi_v = st.vertices.copy(), st.vertices.copy()
            x = st.vertices.ravel()[c]
            lo_v.ravel()[c] = np.float32(x - h)
            hi_v.ravel()[c] = np.float32(x + h)
            span = float(hi_v.ravel()[c]) - float(lo_v.ravel()[c])
            fds.append((loss_at(hi_v) - loss_at(lo_v)) / span)
        if abs(fds[0] - fds[1]) <= max(TOL * max(abs(fds[0]), abs(fds[1])), FLOOR):
            got.append(gv.ravel()[c])
            want.append(fds[0])
    got, want = np.array(got), np.array(want)
    rel_fd = np.linalg.norm(got - want) / np.linalg.norm(want)
    print("vertex gradient: chain rel %.2e; vs FP64 differences on %d of 24 coordinates rel %.2e"
          % (rel_chain, len(got), rel_fd))
    assert len(got) >= 16, len(got)
    assert rel_fd <= 1e-3, rel_fd


def test_rejects_other_formats(ctx, oracle_lib):
    import torch
    from vkhr_gb300._native import VkhrError

    st, b, p, dens, tan, target = diff_scene(oracle_lib, size=(32, 24))
    q = _abi.RaymarchParams.from_buffer_copy(p)
    q.density_format = _abi.DENSITY_U8_UNORM
    buf = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    with pytest.raises(VkhrError) as e:
        ctx.raymarch_train(q, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), None, buf.data_ptr(), 1 << 20, 16)
    assert e.value.status == _abi.VKHR_ERR_NOT_SUPPORTED
    with pytest.raises(VkhrError) as e:
        ctx.raymarch_train(p, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), None, buf.data_ptr(), 16, 16)
    assert e.value.status == _abi.VKHR_ERR_CAPACITY


def test_config_scale_960x540(ctx, oracle_lib):
    """The differentiable workload at full size: the 136,320 x 13 style
    (1,772,160 vertices) splatted into an FP32 256^3 density, FP32 tangents
    from the count voxelizer, 960x540 with 512 steps, 64-step shadows and
    8-tap AO, Kajiya-Kay with kd 0.4, exponents 80 / 8 and shifts +-0.1; the
    target rendered from log-normally perturbed densities (sigma 0.2) with
    first exponent 60.  The gradient is the same for checkpoint intervals 16,
    32 and 64, and matches the FP64 oracle's analytic gradient (relative L2
    1e-3) over the well-conditioned pixels; kd and both exponents match FP64
    central differences of the oracle's loss."""
    import torch

    O = oracle_lib
    from tests._helpers import ill_conditioned, style

    st, t, idx = style("disk", 136_320, 13)
    b = O.bounding_box(st.vertices)
    res = (256, 256, 256)
    n = 256 ** 3
    V = torch.from_numpy(st.vertices).cuda()
    dens = torch.zeros(n, dtype=torch.float32, device="cuda")
    ctx.splat_vertices(V.data_ptr(), st.vertex_count, b, res, dens.data_ptr())
    _, _, tq, _ = O.voxelize("segments", st.vertices, t, idx, b, res)
    tan = np.zeros((n, 4), dtype=np.float32)
    tan[:, :3] = np.maximum(tq[:, :3].astype(np.float32) / 127.0, -1.0)
    kw = dict(camera_distance=4.0, raycast_steps=512.0, shadow_steps=64.0, isosurface=1.0,
              density_format=_abi.DENSITY_F32, tangent_format=_abi.TANGENT_F32X4,
              **{k: v for k, v in scene.CONFIG_SHADING.items() if k != "hair_exponent"})
    p = scene.make_params(b, res, 960, 540, hair_exponent=80.0, **kw)
    pt = scene.make_params(b, res, 960, 540, hair_exponent=60.0, **kw)
    rng = np.random.default_rng(3)
    d_np = dens.cpu().numpy()
    noisy = torch.from_numpy((d_np * rng.lognormal(0.0, 0.2, size=n)).astype(np.float32)).cuda()
    target = torch.empty((540, 960, 4), dtype=torch.float32, device="cuda")
    tdev = torch.from_numpy(tan).cuda()
    ctx.raymarch(pt, noisy.data_ptr(), tdev.data_ptr(), None, target.data_ptr(), None)
    torch.cuda.synchronize()
    tg = target.cpu().numpy()
    # pixels whose outputs hinge on a decision FP32 cannot resolve (the
    # criteria of the raymarch parity tests) are left out of the loss
    # (and, for the tangent gradient, whose normalisation divides by |T|,
    # surface tangents shorter than 0.01)
    ref, _, diag = O.raymarch(p, d_np, tan, diag=True)
    mask = ~ill_conditioned(ref, diag, tangent_floor=1e-2)
    emitted = int((ref[..., 3] > 0).sum())
    assert (~mask).sum() <= 0.02 * emitted + 2, ((~mask).sum(), emitted)
    res_k = [_gpu_grads(ctx, torch, p, d_np, tan, tg, K, mask) for K in (16, 32, 64)]
    for r in res_k[1:]:
        assert np.linalg.norm(r[1] - res_k[0][1]) <= 1e-5 * np.linalg.norm(res_k[0][1])
    loss, gd, gt, gp, rgba = res_k[0]
    assert (rgba[..., 3] > 0).sum() > 10_000
    lref, gd_ref, gt_ref, gp_ref = O.diff_loss(p, d_np.astype(np.float64), tan.astype(np.float64), tg, grads=True,
                                               mask=mask)
    assert abs(loss - lref) <= 1e-4 * lref, (loss, lref)
    for name, g, r in (("density", gd, gd_ref), ("tangent", gt[:, :3], gt_ref[:, :3])):
        rel = np.linalg.norm(g - r) / np.linalg.norm(r)
        print("%s gradient: relative L2 %.2e" % (name, rel))
        assert rel <= 1e-3, (name, rel, int((~mask).sum()), emitted)
    fdp = _fd_params(O, p, d_np.astype(np.float64), tan.astype(np.float64), tg, mask=mask)
    print("kd, exponents: gpu", gp, "oracle", gp_ref, "central differences", fdp)
    assert len(gp) == 3 and all(f is not None for f in fdp), fdp
    assert np.allclose(gp_ref, fdp, rtol=1e-3), (gp_ref, fdp)  # the oracle's own pin at full size
    assert np.allclose(gp, fdp, rtol=1e-3), (gp, fdp)  # the 1e-3 of FP64 central differences
