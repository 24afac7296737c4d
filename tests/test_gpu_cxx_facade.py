"""The C++17 facade (include/vkhr/cuda.hh), compiled with g++ against
libvkhr_cuda.so, voxelizes, raymarches and resolves the colour pass like the
reference's host would; its outputs must equal the oracle's (voxels and
resolved frames bit-exact, the raymarched image within the raymarch
tolerance)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from vkhr_gb300 import _abi, _native, scene, workloads
from tests._helpers import background_case, build_ppll, image_errors, style

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.gpu


def test_cxx_facade(native_lib, oracle_lib, tmp_path):
    exe = tmp_path / "facade_test"
    libdir = os.path.dirname(_native.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests/cxx/facade_test.cc"),
           "-L", libdir, "-l:libvkhr_cuda.so", "-Wl,-rpath," + libdir, "-o", str(exe)]
    subprocess.run(cmd, check=True)
    st, t, idx = style("hemi", 3000, 12, seed=9)
    res = (40, 36, 44)
    b = oracle_lib.bounding_box(st.vertices)
    p = scene.make_params(b, res, 96, 72, raycast_steps=128.0)
    # compositing inputs: rasterizer-like strand fragments, a background, and
    # the PPLL those fragments build when linked in order
    f = workloads.strand_fragments(st.vertices, t, idx, p, 0.5, "cpu").numpy().view(_abi.FRAGMENT_DTYPE).reshape(-1)
    bg = background_case(96, 72, 31)
    heads, nodes = build_ppll(f, 96, 72, seed=32)
    blob = (np.array([st.vertex_count, idx.shape[0]], np.uint32).tobytes() + np.array(res, np.int32).tobytes()
            + bytes(b) + st.vertices.tobytes() + t.tobytes() + idx.tobytes() + bytes(p)
            + np.uint32(len(f)).tobytes() + f.tobytes() + bg.tobytes() + np.uint32(len(nodes)).tobytes()
            + heads.tobytes() + nodes.tobytes())
    (tmp_path / "in.bin").write_bytes(blob)
    out = str(tmp_path / "o")
    r = subprocess.run([str(exe), str(tmp_path / "in.bin"), out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    n = res[0] * res[1] * res[2]
    for mode, tag in (("vertices", "v"), ("segments", "s")):
        c, d, tq, _ = oracle_lib.voxelize(mode, st.vertices, t, idx, b, res)
        assert np.array_equal(np.fromfile(out + "_%s_dens.bin" % tag, np.uint8), d)
        assert np.array_equal(np.fromfile(out + "_%s_tan.bin" % tag, np.int8).reshape(n, 4), tq)
        if tag == "s":
            assert np.array_equal(np.fromfile(out + "_s_counts.bin", np.uint32), c)
            dn = oracle_lib.normalize(d)
            assert np.array_equal(np.fromfile(out + "_s_norm.bin", np.uint8), dn)
            ref, rdepth, diag = oracle_lib.raymarch(p, dn, tq, diag=True)
            gpu = np.fromfile(out + "_rgba.bin", np.float32).reshape(72, 96, 4)
            rms, mx, excluded, emitted = image_errors(gpu, ref, diag)
            assert emitted > 0 and np.all(rms <= 1e-3) and np.all(mx <= 2e-2)
    # LinkedList: resolve.comp over the lists, and the PPLL-free composite over
    # the facade's own raymarched image, both bit-exact
    ppll = np.fromfile(out + "_ppll.bin", np.uint32).reshape(72, 96)
    rc, want = oracle_lib.resolve_ppll(heads, nodes, bg)
    assert rc == 0 and np.array_equal(ppll, want)
    comp = np.fromfile(out + "_composite.bin", np.uint32).reshape(72, 96)
    vdepth = np.fromfile(out + "_depth.bin", np.float32).reshape(72, 96)
    vrgba = np.fromfile(out + "_rgba.bin", np.float32).reshape(72, 96, 4)
    assert np.array_equal(comp, oracle_lib.composite(f, bg, vrgba, vdepth))
