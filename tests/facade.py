"""Build helper for the C++ facade test program (tests/cpp/facade_main.cpp):
compiled with g++ against include/pisurf.hpp and linked to the library."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")
BIN = os.path.join(OUT, "facade_main")


def build():
    from particleisosurface_gb300 import build as B
    lib = B.build()
    libdir = os.path.dirname(lib)
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "cpp", "facade_main.cpp")
    if os.path.exists(BIN) and os.path.getmtime(BIN) > max(
            os.path.getmtime(src), os.path.getmtime(lib),
            os.path.getmtime(os.path.join(ROOT, "include", "pisurf.hpp"))):
        return BIN
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I" + os.path.join(ROOT, "include"), src,
           "-L" + libdir, "-lpisurf", "-Wl,-rpath," + libdir, "-o", BIN]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("facade build failed:\n" + r.stdout + r.stderr)
    return BIN
