"""The FP64 oracle of the differentiable path against FP64 central finite
differences (h = 1e-3): the analytic gradient with respect to densities,
tangent components, kd and the specular exponents, and the splat's adjoint;
for the reference's shading, for the workloads' dual-lobe Kajiya-Kay with
tangent shifts, and for the directional ambient occlusion.
A coordinate is ill-conditioned, and excluded (at most 10% of them), when
the loss is not smooth there at the scale of h: the central differences
at h and h/2 disagree by more than 1e-3 relative, or the loss at the point
departs from the mean of its neighbours at +-h by as much at h/2 as at h
(a jump at the point; a smooth loss departs by h^2 f'' / 2).
Densities are checked at voxels of nonzero density: at a zero voxel the
shader's `density != 0` test makes the loss discontinuous at the point
itself, and the gradient there is that of the branch the point takes."""
import numpy as np
import pytest

from vkhr_gb300 import _abi, scene
from tests._helpers import style

H = 1e-3
TOL = 1e-3
FLOOR = 1e-10  # |dL/dx| below this is rounding noise of the loss (~1e-16 L / h)


SHADINGS = {
    "reference": {},
    "dual_lobe": {"spec_exponent2": 8.0, "spec_shift": (0.1, -0.1)},
    "dual_lobe_ao16": {"spec_exponent2": 8.0, "spec_shift": (0.1, -0.1), "ao_directions": 16},
}


def diff_scene(O, res=(24, 24, 24), size=(40, 30), steps=64.0, seed=3, shading=None):
    """A splatted style, a smooth random tangent field, and a target image
    rendered from log-normally perturbed densities with exponent 60."""
    st, t, idx = style("hemi", 1500, 12, seed=seed)
    b = O.bounding_box(st.vertices)
    n = res[0] * res[1] * res[2]
    dens = O.splat(st.vertices, b, res)
    rng = np.random.default_rng(seed)
    tan = np.zeros((n, 4))
    tan[:, :3] = np.array([1.0, 0.3, 0.2]) + 0.3 * rng.normal(size=(n, 3))
    kw = dict(camera_distance=5.0, raycast_steps=steps, shadow_steps=32.0, isosurface=1.0, kd=0.4,
              density_format=_abi.DENSITY_F32, tangent_format=_abi.TANGENT_F32X4, **(shading or {}))
    p = scene.make_params(b, res, size[0], size[1], hair_exponent=80.0, **kw)
    pt = scene.make_params(b, res, size[0], size[1], hair_exponent=60.0, **kw)
    noisy = (dens * rng.lognormal(0.0, 0.2, size=n)).astype(np.float32)
    target, _ = O.raymarch(pt, noisy, tan.astype(np.float32))
    return st, b, p, dens, tan, target


def central(f, x0, h):
    """(f(x0 + h) - f(x0 - h)) / 2h and |f(x0) - mean(f(x0 - h), f(x0 + h))|."""
    lo, mid, hi = f(x0 - h), f(x0), f(x0 + h)
    return (hi - lo) / (2 * h), abs(mid - 0.5 * (lo + hi))


def check(fd_of, analytic, coords):
    bad, ill = [], 0
    for c in coords:
        (f1, dev1), (f2, dev2) = fd_of(c, H), fd_of(c, H / 2)
        jump = dev1 > 1e-13 and dev2 > 0.5 * dev1
        if jump or abs(f1 - f2) > max(TOL * max(abs(f1), abs(f2)), FLOOR):
            ill += 1
            continue
        a = analytic(c)
        if abs(a - f1) > max(TOL * abs(f1), FLOOR):
            bad.append((c, a, f1))
    assert ill <= 0.1 * len(coords), ill
    assert not bad, bad[:5]


@pytest.mark.parametrize("shading", sorted(SHADINGS))
def test_density_tangent_and_params(oracle_lib, shading):
    O = oracle_lib
    st, b, p, dens, tan, target = diff_scene(O, shading=SHADINGS[shading])
    loss, gd, gt, gp = O.diff_loss(p, dens, tan, target, grads=True)
    assert np.abs(gd).max() > 0 and np.abs(gt).max() > 0
    rng = np.random.default_rng(1)
    touched = np.nonzero((gd != 0) & (dens > 0))[0]
    dcoords = rng.choice(touched, size=48, replace=False)

    def fd_density(i, h):
        def f(x):
            d = dens.copy()
            d[i] = x
            return O.diff_loss(p, d, tan, target)
        return central(f, dens[i], h)

    check(fd_density, lambda i: gd[i], dcoords)

    ttouched = np.nonzero(np.abs(gt[:, :3]).sum(axis=1))[0]
    tcoords = [(int(v), int(k)) for v, k in zip(rng.choice(ttouched, size=24, replace=False), rng.integers(0, 3, 24))]

    def fd_tangent(ck, h):
        v, k = ck
        def f(x):
            t2 = tan.copy()
            t2[v, k] = x
            return O.diff_loss(p, dens, t2, target)
        return central(f, tan[v, k], h)

    check(fd_tangent, lambda ck: gt[ck[0], ck[1]], tcoords)

    def fd_param(k, h):
        # the parameter block holds float32: difference over the stored values
        field = ("kd", "hair_exponent", "spec_exponent2")[k]

        def at(x):
            q = _abi.RaymarchParams.from_buffer_copy(p)
            setattr(q, field, x)
            return q, getattr(q, field)
        x0 = getattr(p, field)
        (qm, xm), (qp, xp) = at(x0 - h), at(x0 + h)
        lo, mid, hi = (O.diff_loss(q, dens, tan, target) for q in (qm, p, qp))
        return (hi - lo) / (xp - xm), abs(mid - (lo * (xp - x0) + hi * (x0 - xm)) / (xp - xm))

    check(fd_param, lambda k: gp[k], [0, 1, 2] if p.spec_exponent2 > 0 else [0, 1])
    if p.spec_exponent2 <= 0:
        assert gp[2] == 0


def test_splat_adjoint(oracle_lib):
    """d(sum g * splat(V)) / dV against central differences of vertex coordinates."""
    O = oracle_lib
    st, t, idx = style("disk", 300, 10, seed=4)
    b = O.bounding_box(st.vertices)
    res = (20, 18, 22)
    rng = np.random.default_rng(2)
    g = rng.normal(size=res[0] * res[1] * res[2])
    gv = O.splat_adjoint(st.vertices, b, res, g)
    skipped = 0
    for i, k in zip(rng.integers(0, st.vertex_count, 32), rng.integers(0, 3, 32)):
        def f(x):
            v = st.vertices.astype(np.float64).copy()
            v[i, k] = x
            return float(np.dot(g, O.splat(v.astype(np.float32), b, res)))
        # float32 vertices: steps that are exact in float32; the splat is
        # linear along an axis between texel centres
        x0 = float(st.vertices[i, k])
        fd1 = (f(x0 + 2.0 ** -12) - f(x0 - 2.0 ** -12)) / 2.0 ** -11
        fd2 = (f(x0 + 2.0 ** -13) - f(x0 - 2.0 ** -13)) / 2.0 ** -12
        if abs(fd1 - fd2) > 1e-6 * max(1.0, abs(fd1)):  # a texel centre within the step
            skipped += 1
            continue
        assert abs(fd1 - gv[i, k]) <= 1e-6 * max(1.0, abs(fd1)), (i, k, fd1, gv[i, k])
    assert skipped <= 3


@pytest.mark.parametrize("shading", sorted(SHADINGS))
def test_forward_matches_raymarch_oracle(oracle_lib, shading):
    """The differentiable oracle's forward is the FP64 raymarch oracle
    (volume.frag:31-103): with that oracle's image as the target the loss is
    only the rounding of the target to float32."""
    O = oracle_lib
    st, b, p, dens, tan, target = diff_scene(O, shading=SHADINGS[shading])
    d32, t32 = dens.astype(np.float32), tan.astype(np.float32)
    ref, _ = O.raymarch(p, d32, t32, precision="f64")
    assert (ref[..., 3] > 0).sum() > 100
    assert O.diff_loss(p, d32.astype(np.float64), t32.astype(np.float64), ref) < 1e-9
