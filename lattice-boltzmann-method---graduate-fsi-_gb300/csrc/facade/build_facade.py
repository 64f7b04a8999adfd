"""Build the C++ drop-in facade (LBM.h) drivers against liblbmgpu.so.

Each driver in DRIVERS is compiled together with lbm_facade.cpp (with the
reference compile-time switches of DRIVER_FLAGS) and linked with -llbmgpu
(rpath to the package directory) into csrc/facade/_build/.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "_build")
DRIVERS = ["dropin_cavity", "dropin_sphere", "dropin_sphere_bb", "dropin_details", "dropin_cylinder2d",
           "dropin_couette", "dropin_staircase2d", "dropin_poiseuille", "dropin_rayleigh"]
# compile-time switches of the reference a driver is built with
DRIVER_FLAGS = {"dropin_details": ["-DMORE_DETAILS"], "dropin_cylinder2d": ["-DD2Q9"],
                "dropin_couette": ["-DD2Q9", "-DENERGY"], "dropin_staircase2d": ["-DD2Q9"],
                "dropin_poiseuille": ["-DD2Q9", "-DENERGY"], "dropin_rayleigh": ["-DENERGY"]}


def build(force: bool = False) -> list:
    os.makedirs(OUT, exist_ok=True)
    lib = os.path.join(PKG, "liblbmgpu.so")
    srcs = [os.path.join(HERE, f) for f in ("lbm_facade.cpp", "LBM.h")]
    outs = []
    for d in DRIVERS:
        exe = os.path.join(OUT, d)
        deps = srcs + [os.path.join(HERE, d + ".cpp"), lib]
        if force or not os.path.exists(exe) or any(os.path.getmtime(p) > os.path.getmtime(exe) for p in deps):
            cmd = ["g++", "-O2", "-std=c++17", "-I" + HERE] + DRIVER_FLAGS.get(d, []) + [os.path.join(HERE, d + ".cpp"),
                   os.path.join(HERE, "lbm_facade.cpp"), "-L" + PKG, "-llbmgpu",
                   "-Wl,-rpath," + PKG, "-o", exe]
            subprocess.check_call(cmd)
        outs.append(exe)
    return outs


if __name__ == "__main__":
    print(build(force=True))
