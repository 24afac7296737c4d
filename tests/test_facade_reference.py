"""The C++ facade against the reference's own HairStyle type: the
voxelize_* templates compile for vkhr::HairStyle (include/vkhr/scene_graph/
hair_style.hh, with glm from oracle/glmshim), and to_reference yields the
reference's HairStyle::Volume field for field, so that the loader's call
site (src/vkhr/rasterizer/hair_style.cc:75) changes in one line.  Host-only;
skipped where the reference sources are not present."""
import os
import subprocess

import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cxx", "reference_volume_test.cc")
REF_HEADER = os.path.join(O.REFERENCE_ROOT, "include", "vkhr", "scene_graph", "hair_style.hh")

pytestmark = pytest.mark.skipif(not os.path.isfile(REF_HEADER), reason="the reference sources are not present")


def _cmd(*extra):
    return ["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"), "-I",
            os.path.join(ROOT, "oracle", "glmshim"), "-I", os.path.join(O.REFERENCE_ROOT, "include"), *extra]


def test_facade_templates_compile_for_reference_hairstyle(tmp_path):
    subprocess.run(_cmd("-c", SRC, "-o", str(tmp_path / "t.o")), check=True)


def test_to_reference_volume(tmp_path):
    exe = tmp_path / "conv"
    subprocess.run(_cmd("-DVKHR_CONVERSION_ONLY", SRC, "-o", str(exe)), check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
