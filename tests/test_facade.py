"""The C++ facade (include/pisurf.hpp): a host program written against the
reference's class names compiles, links to the library and, without a GPU,
fails with the library's CUDA error instead of computing on the CPU."""
import json
import subprocess

import numpy as np

import facade
from conftest import HAS_GPU
from particleisosurface_gb300 import synth


def test_facade_program_builds_and_reports_no_cpu_fallback(tmp_path):
    exe = facade.build()
    fr = synth.small_blob(n=500, seed=5)
    src = tmp_path / "xyz.f32"
    fr.xyz.astype(np.float32).tofile(src)
    r = subprocess.run([exe, str(src), str(fr.n), repr(fr.radius), str(tmp_path / "out.obj")],
                       capture_output=True, text=True, timeout=120)
    line = json.loads(r.stdout.strip().splitlines()[-1])
    if HAS_GPU:
        assert r.returncode == 0, r.stdout + r.stderr
        assert line["vertices"] > 0
    else:
        assert r.returncode == 3, r.stdout + r.stderr
        assert line["error"] == -2
