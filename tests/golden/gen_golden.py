"""Generate the golden fixtures in tests/golden/ from the reference itself.

The reference's own lbm.cpp is compiled unmodified by oracle/build_ref.sh
(with oracle/ref_config.h and oracle/ref_harness.cpp) and run here; its
outputs are stored as small .npz fixtures:

  cavity12_tau0.8_lid0.05_200.npz   D3Q19 lid-driven cavity 12^3, 200 steps:
                                    full interior rho, ux, uy, uz
  cavity12_vtk_200.npz              the same run's OutputVTK file
  cylinder80x40_vtk_100.npz         the D2Q9 cylinder's OutputVTK and OutputVTK_Marker files
                                    (lbm.cpp:2290-2642): header text and
                                    every appended array
  cavity64_tau0.8_lid0.05_5000.npz  the 64^3, tau = 0.8, 5000-step cavity:
                                    mid planes k = 32 and i = 32 of rho, u,
                                    plus interior sums and maxima
  cylinder80x40_D10_n40_m5_100.npz  D2Q9 implicit-IBM cylinder (the shipped
                                    default case shrunk): rho, ux, uy, Fx, Fy
                                    on the k = 1 layer, Cl and Cd per step
  sphere_bb48x24x24_D8_Re20_100.npz  D3Q19 staircase sphere (the Sphere_BB
                                    case shrunk, u = 0.05): mid planes
                                    k = 12 and j = 12 of rho, u, interior
                                    sums and maxima, momentum-exchange Cl
                                    and Cd after every step
  cylinder80x40_D10_n40_explicit_100.npz  the same cylinder with the
                                    explicit direct-forcing scheme (run on
                                    one thread: the reference's drag sum is
                                    an unsynchronised OpenMP update)
  cylinder80x40_D10_n40_m5_transverse_100.npz  the cylinder oscillating
                                    across the stream
                                    (Cylinder_Transverse_Oscillation, A = 2,
                                    f = 0.005, u = 0.05, Re = 100)
  couette_energy_ny30_re20_2000.npz  D2Q9 Couette flow with the reference's
                                    own thermal model (ENERGY), Ny = 30,
                                    Re = 20, 2000 steps: rho, u, T and the
                                    heat flux q on every row of the k = 1
                                    layer, ghosts included
  cylinder80x40_D10_n40_m5_inline_100.npz  the cylinder oscillating along the
                                    stream in fluid at rest
                                    (Cylinder_Inline_Oscillating, KC = 5,
                                    period 1000 steps, centre (Nx/2, Ny/2))
  cylinder120x40_D10_n40_m5_towed_100.npz  the cylinder towed at -0.1
                                    through fluid at rest
                                    (Cylinder_IBM_Moving_Arbie, centre x = 80)
  poiseuille_ny30_re20{,_energy}_1500.npz  the body-forced channel
                                    (Poiseuille_Flow, Ny = 30, Re = 20), with
                                    and without the ENERGY model: rho, u (and
                                    T, q) of every row of the k = 1 layer
  staircase2d_{cylbasic,tandem,triangle}_300.npz  the D2Q9 staircase bodies
                                    with momentum-exchange Cl/Cd
                                    (Cylinder_Basic, Cylinder_Tandem_Circle,
                                    Cylinder_Tandem_Triangle, shrunk): Cl and
                                    Cd of every body after every step, the
                                    set-up's cell types, a window of rho, u
                                    round the bodies and the layer sums
                                    These two keep Cl, Cd, the markers, and
                                    rho, u, F in the IBM box window
                                    i = 4..28, j = 8..32 of the k = 1 layer
                                    plus sums over the whole layer
  cavity8_details_200.npz           the 8^3 cavity (tau = 0.8, lid 0.05)
                                    built in MORE_DETAILS mode, 200 steps,
                                    Sup_MacroProp every 10 steps: every
                                    cell (ghosts included) of rho, u,
                                    pressure, the 6 distinct viscous
                                    stresses, the running averages and rms
                                    values; and that run's OutputVTK file
                                    (vtk_* keys)

Run from the repository root:  python tests/golden/gen_golden.py
(needs the reference tree; the 64^3 case takes a few minutes on 8 cores;
--cav64-dump PATH reuses a dump the harness already wrote).
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(ROOT, "oracle", "_ref")


def read_vtr(path: str) -> dict:
    """Header text and every appended DataArray of a RectilinearGrid file."""
    import re

    raw = open(path, "rb").read()
    cut = raw.index(b'<AppendedData encoding="raw">') + len(b'<AppendedData encoding="raw">')
    head = raw[:cut].decode()
    data = raw[cut + 1:]
    out = {"header": np.array(head)}
    for m in re.finditer(r'Name="([^"]+)"(?: NumberOfComponents="(\d+)")? format="appended" offset="(\d+)"', head):
        off = int(m.group(3))
        n = int(np.frombuffer(data[off:off + 4], dtype=np.uint32)[0])
        out[m.group(1)] = np.frombuffer(data[off + 4:off + 4 + n], dtype=np.float32).copy()
    return out


# (name, build_ref variant, executable, nx, ny, bodies, window rows, window columns)
STAIRCASE = (("cylbasic", "cylbasic:100:60:20:200:0.1", "ref_cylbasic_100_60_20_200_0.1", 100, 60, 1,
              slice(14, 48), slice(4, 50)),
             ("tandem", "tandem:160:100:10:100:0.05:1.5:2", "ref_tandem_160_100_10_100_0.05_1.5_2", 160, 100, 2,
              slice(24, 72), slice(16, 60)),
             ("triangle", "triangle:100:80:10:100:0.05:1.5:3", "ref_triangle_100_80_10_100_0.05_1.5_3", 100, 80, 3,
              slice(26, 56), slice(14, 92)))
STAIRCASE_VARIANTS = tuple(v for _, v, *_ in STAIRCASE)


def cylinder_vtk(tmp: str) -> None:
    """The shipped D2Q9 implicit-IBM cylinder (80 x 40, D = 10, 40 markers,
    m_max = 5), 100 steps, with the reference's own OutputVTK file of the
    final state and its OutputVTK_Marker file."""
    import glob

    p = os.path.join(tmp, "cylvtk.bin")
    subprocess.check_call([os.path.join(REF, "ref_cylinder_80_40_10_40_5"), "100", p, "vtk"], cwd=tmp)
    v = read_vtr(os.path.join(tmp, "field000000.vtr"))
    wall = glob.glob(os.path.join(tmp, "wall_t*.vtk"))
    assert len(wall) == 1, wall
    v["marker_file"] = open(wall[0]).read()
    v["marker_file_name"] = os.path.basename(wall[0])
    np.savez_compressed(os.path.join(OUT, "cylinder80x40_vtk_100.npz"), steps=100, **v)


def triangle_details(tmp: str) -> None:
    """The reference's Cylinder_Tandem_Triangle in MORE_DETAILS mode (D2Q9,
    60 x 40, D = 10, two triangles 1.5 D apart, Re = 100, u = 0.05), 200
    steps with Sup_MacroProp every Nt = 10: the k = 1 layer of rho, u, the
    pressure, the viscous stress and the running statistics, the
    momentum-exchange Cl / Cd of both bodies after every step, the cell
    types, and the reference's own OutputVTK and OutputAVGVTK files."""
    nx, ny, nb, steps = 60, 40, 2, 200
    d = os.path.join(tmp, "trid")
    os.makedirs(d)
    p, pt = os.path.join(d, "tri.bin"), os.path.join(d, "tri.types")
    subprocess.check_call([os.path.join(REF, "ref_triangled_60_40_10_100.0_0.05_1.5_2"), str(steps), p, pt, "vtk"],
                          cwd=d)
    n3 = (nx + 2) * (ny + 2) * 3
    a = np.fromfile(p)
    f4 = a[:4 * n3].reshape(4, 3, ny + 2, nx + 2)[:, 1]
    rest = a[4 * n3:4 * n3 + nb * 2 * steps].reshape(nb, 2, steps)
    det = a[4 * n3 + nb * 2 * steps:].reshape(36, 3, ny + 2, nx + 2)[:, 1]
    # details order: pressure, sigma[3][3], avg_velocity, avg_pressure,
    # avg_ReynoldStress, rms_velocity, rms_pressure, rms_ReynoldStress
    sym = {}
    for base, name in ((1, "sigma"), (14, "avg_rs"), (27, "rms_rs")):
        t = det[base:base + 9].reshape(3, 3, ny + 2, nx + 2)
        for i in range(3):
            for j in range(i):
                assert np.array_equal(t[i, j], t[j, i]), (name, i, j)
        sym[name] = np.stack([t[0, 0], t[0, 1], t[0, 2], t[1, 1], t[1, 2], t[2, 2]])
    base = os.path.join(d, "output Tandem Triangle", "LpD = 1.5 Re = 100")
    v = read_vtr(os.path.join(base, "Flowfield", "field000000.vtr"))
    w = read_vtr(os.path.join(base, "avgfield.vtr"))
    types = np.fromfile(pt, dtype=np.uint8).reshape(ny + 2, nx + 2)
    np.savez_compressed(os.path.join(OUT, "triangle60x40_details_200.npz"), rho=f4[0], u=f4[1:4], p=det[0],
                        sigma=sym["sigma"], avg_u=det[10:13], avg_p=det[13], avg_rs=sym["avg_rs"],
                        rms_u=det[23:26], rms_p=det[26], rms_rs=sym["rms_rs"], cl=rest[:, 0], cd=rest[:, 1],
                        types=types, nx=nx, ny=ny, D=10, Re=100.0, u_in=0.05, lpd=1.5, nb=nb, steps=steps, nt=10,
                        **{"vtk_" + k: x for k, x in v.items()}, **{"avgvtk_" + k: x for k, x in w.items()})


def couette_neumann(tmp: str) -> None:
    """The ENERGY Couette flow with its top wall a Neumann wall (j.n = 0),
    1000 steps.  The reference evaluates Neumann walls inside its push, so
    its result depends on the order its OpenMP threads visit the cells; one
    thread gives the serial order the oracle and the device restate."""
    p = os.path.join(tmp, "couette_neumann.bin")
    env = dict(os.environ, OMP_NUM_THREADS="1")
    subprocess.check_call([os.path.join(REF, "ref_couette_30_20_neumann"), "1000", p], env=env)
    f = oracle.read_ref_dump(p, 4, 32, 4, 8)["fields"]
    for k in range(4):
        assert np.array_equal(f[:, k], f[:, 1])
    np.savez_compressed(os.path.join(OUT, "couette_neumann_ny30_re20_1000.npz"), rho=f[0, 1], u=f[1:4, 1],
                        T=f[4, 1], q=f[5:8, 1], ny=30, Re=20.0, steps=1000)


def rayleigh(tmp: str) -> None:
    """The reference's Rayleigh_Benard case (D3Q19 ENERGY: Dirichlet y
    walls, Neumann x and z walls, buoyancy) on a 32 x 16 x 5 box, 400 steps,
    on one thread (its Neumann walls make the result depend on the visiting
    order).  Every cell, ghosts included: rho, u, F, T, q."""
    p = os.path.join(tmp, "rayleigh.bin")
    env = dict(os.environ, OMP_NUM_THREADS="1")
    subprocess.check_call([os.path.join(REF, "ref_rayleigh_32_16_5"), "400", p], env=env)
    f = oracle.read_ref_dump(p, 34, 18, 7, 11)["fields"]
    np.savez_compressed(os.path.join(OUT, "rayleigh32x16x5_400.npz"), rho=f[0], u=f[1:4], F=f[4:7], T=f[7],
                        q=f[8:11], nx=32, ny=16, nz=5, steps=400)


def run(exe: str, args: list[str]) -> None:
    subprocess.check_call([os.path.join(REF, exe)] + args)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--cav64-dump", default=None)
    ap.add_argument("--skip-cav64", action="store_true")
    ap.add_argument("--only-cylinder-vtk", action="store_true",
                    help="write only cylinder80x40_vtk_100.npz (the D2Q9 OutputVTK / OutputVTK_Marker files)")
    ap.add_argument("--only-couette-neumann", action="store_true",
                    help="write only couette_neumann_ny30_re20_1000.npz (the ENERGY Couette, Neumann top wall)")
    ap.add_argument("--only-rayleigh", action="store_true",
                    help="write only rayleigh32x16x5_400.npz (D3Q19 ENERGY, Rayleigh-Benard)")
    ap.add_argument("--only-triangle-details", action="store_true",
                    help="write only triangle60x40_details_200.npz (D2Q9 MORE_DETAILS, both VTK files)")
    a = ap.parse_args()
    if a.only_couette_neumann:
        oracle.build_ref("couette:30:20:neumann")
        couette_neumann(tempfile.mkdtemp())
        return
    if a.only_rayleigh:
        oracle.build_ref("rayleigh:32:16:5")
        rayleigh(tempfile.mkdtemp())
        return
    if a.only_triangle_details:
        oracle.build_ref("triangled:60:40:10:100.0:0.05:1.5:2")
        triangle_details(tempfile.mkdtemp())
        return
    if a.only_cylinder_vtk:
        oracle.build_ref("cylinder:80:40:10:40:5")
        cylinder_vtk(tempfile.mkdtemp())
        return
    oracle.build_ref("cavity:12:0.8", "cavity:64:0.8", "cylinder:80:40:10:40:5", "sphere:48:24:24:8:20:0.05",
                     "details:8:0.8", "explicit:80:40:10:40", "transverse:80:40:10:40:5:2.0:0.005",
                     "couette:30:20", "couette:30:20:neumann", "inline:80:40:10:40:5:1000", "arbie:120:40:10:40:5:80", "poiseuille:30:20",
                     "poiseuille:30:20:energy", "triangled:60:40:10:100.0:0.05:1.5:2", "rayleigh:32:16:5",
                     *STAIRCASE_VARIANTS)
    tmp = tempfile.mkdtemp()

    # 12^3 cavity, 200 steps (and the reference's own VTK file of it)
    p = os.path.join(tmp, "cav12.bin")
    subprocess.check_call([os.path.join(REF, "ref_cavity_12_0.8"), "200", p, "0.05", "vtk"], cwd=tmp)
    v = read_vtr(os.path.join(tmp, "field000000.vtr"))
    np.savez_compressed(os.path.join(OUT, "cavity12_vtk_200.npz"), **v)
    f = oracle.read_ref_dump(p, 14, 14, 14, 4)["fields"][:, 1:-1, 1:-1, 1:-1]
    np.savez_compressed(os.path.join(OUT, "cavity12_tau0.8_lid0.05_200.npz"), rho=f[0], ux=f[1], uy=f[2], uz=f[3],
                        n=12, tau=0.8, lid=0.05, steps=200)

    # 64^3 cavity, 5000 steps
    if not a.skip_cav64:
        p = a.cav64_dump or os.path.join(tmp, "cav64.bin")
        if not a.cav64_dump:
            run("ref_cavity_64_0.8", ["5000", p, "0.05"])
        f = oracle.read_ref_dump(p, 66, 66, 66, 4)["fields"][:, 1:-1, 1:-1, 1:-1]
        np.savez_compressed(os.path.join(OUT, "cavity64_tau0.8_lid0.05_5000.npz"),
                            zmid=f[:, 32, :, :], xmid=f[:, :, :, 32], sums=f.reshape(4, -1).sum(axis=1),
                            absmax=np.abs(f.reshape(4, -1)).max(axis=1), n=64, tau=0.8, lid=0.05, steps=5000)

    # 2D implicit IBM cylinder, 100 steps
    p = os.path.join(tmp, "cyl.bin")
    steps = 100
    run("ref_cylinder_80_40_10_40_5", [str(steps), p])
    r = oracle.read_ref_dump(p, 82, 42, 3, 7, steps, 40)
    fl = r["fields"][:, 1]  # k = 1 layer
    np.savez_compressed(os.path.join(OUT, "cylinder80x40_D10_n40_m5_100.npz"), rho=fl[0], ux=fl[1], uy=fl[2],
                        Fx=fl[4], Fy=fl[5], cl=r["cl"], cd=r["cd"], markers=r["markers"], nx=80, ny=40, D=10.0,
                        nodes=40, m_max=5, steps=steps)
    # staircase sphere with momentum exchange, 100 steps
    p = os.path.join(tmp, "sph.bin")
    steps = 100
    run("ref_sphere_48_24_24_8_20_0.05", [str(steps), p])
    r = oracle.read_ref_dump(p, 50, 26, 26, 4, steps, 0)
    f = r["fields"][:, 1:-1, 1:-1, 1:-1]
    np.savez_compressed(os.path.join(OUT, "sphere_bb48x24x24_D8_Re20_100.npz"), zmid=f[:, 12, :, :],
                        ymid=f[:, :, 12, :], sums=f.reshape(4, -1).sum(axis=1),
                        absmax=np.abs(f.reshape(4, -1)).max(axis=1), cl=r["cl"], cd=r["cd"], nx=48, ny=24, nz=24,
                        D=8.0, Re=20.0, u=0.05, steps=steps)
    # 2D cylinders: explicit scheme, transverse oscillation (100 steps)
    for exe, name, env in (("ref_explicit_80_40_10_40", "cylinder80x40_D10_n40_explicit_100.npz", {"OMP_NUM_THREADS": "1"}),
                           ("ref_transverse_80_40_10_40_5_2.0_0.005", "cylinder80x40_D10_n40_m5_transverse_100.npz", {})):
        p = os.path.join(tmp, name + ".bin")
        subprocess.check_call([os.path.join(REF, exe), "100", p], env=dict(os.environ, **env))
        r = oracle.read_ref_dump(p, 82, 42, 3, 7, 100, 40)
        fl = r["fields"][:, 1]  # k = 1 layer, [field][j][i]
        np.savez_compressed(os.path.join(OUT, name), window=fl[[0, 1, 2, 4, 5], 8:33, 4:29],
                            sums=fl[[0, 1, 2, 4, 5]].reshape(5, -1).sum(axis=1), cl=r["cl"], cd=r["cd"],
                            markers=r["markers"], nx=80, ny=40, D=10.0, nodes=40, steps=100)

    # moving bodies in fluid at rest: inline oscillation, towed cylinder (100 steps)
    for exe, name, nx in (("ref_inline_80_40_10_40_5_1000", "cylinder80x40_D10_n40_m5_inline_100.npz", 80),
                          ("ref_arbie_120_40_10_40_5_80", "cylinder120x40_D10_n40_m5_towed_100.npz", 120)):
        p = os.path.join(tmp, name + ".bin")
        run(exe, ["100", p])
        r = oracle.read_ref_dump(p, nx + 2, 42, 3, 7, 100, 40)
        fl = r["fields"][:, 1]
        np.savez_compressed(os.path.join(OUT, name), window=fl[[0, 1, 2, 4, 5], 6:36, nx // 2 - 20:nx // 2 + 30],
                            sums=fl[[0, 1, 2, 4, 5]].reshape(5, -1).sum(axis=1), cl=r["cl"], cd=r["cd"],
                            markers=r["markers"], nx=nx, ny=40, D=10.0, nodes=40, steps=100)

    # MORE_DETAILS cavity, 200 steps (averages sampled every Nt = 10 steps)
    d = os.path.join(tmp, "det")
    os.makedirs(d)
    p = os.path.join(d, "det.bin")
    subprocess.check_call([os.path.join(REF, "ref_details_8_0.8"), "200", p, "0.05", "vtk"], cwd=d)
    # dump order: rho, u, then pressure, sigma[3][3], avg_velocity,
    # avg_pressure, avg_ReynoldStress, rms_velocity, rms_pressure,
    # rms_ReynoldStress
    f = oracle.read_ref_dump(p, 10, 10, 10, 40)["fields"]
    sym = {}
    for base, name in ((5, "sigma"), (18, "avg_rs"), (31, "rms_rs")):
        t = f[base:base + 9].reshape(3, 3, 10, 10, 10)
        for a in range(3):
            for b in range(a):
                assert np.array_equal(t[a, b], t[b, a]), (name, a, b)
        sym[name] = np.stack([t[0, 0], t[0, 1], t[0, 2], t[1, 1], t[1, 2], t[2, 2]])
    v = read_vtr(os.path.join(d, "field000000.vtr"))
    np.savez_compressed(os.path.join(OUT, "cavity8_details_200.npz"), rho=f[0], u=f[1:4], p=f[4],
                        sigma=sym["sigma"], avg_u=f[14:17], avg_p=f[17], avg_rs=sym["avg_rs"], rms_u=f[27:30],
                        rms_p=f[30], rms_rs=sym["rms_rs"], n=8, tau=0.8, lid=0.05, steps=200, nt=10,
                        **{"vtk_" + k: a for k, a in v.items()})
    # ENERGY Couette flow, 2000 steps: every k layer evolves alike (cz = 0)
    p = os.path.join(tmp, "couette.bin")
    run("ref_couette_30_20", ["2000", p])
    f = oracle.read_ref_dump(p, 4, 32, 4, 8)["fields"]
    for k in range(4):
        assert np.array_equal(f[:, k], f[:, 1])
    np.savez_compressed(os.path.join(OUT, "couette_energy_ny30_re20_2000.npz"), rho=f[0, 1], u=f[1:4, 1],
                        T=f[4, 1], q=f[5:8, 1], ny=30, Re=20.0, steps=2000)
    couette_neumann(tmp)
    rayleigh(tmp)
    # Poiseuille channel, 1500 steps, with and without ENERGY
    for exe, name, nf in (("ref_poiseuille_30_20", "poiseuille_ny30_re20_1500.npz", 4),
                          ("ref_poiseuille_30_20_energy", "poiseuille_ny30_re20_energy_1500.npz", 8)):
        p = os.path.join(tmp, name + ".bin")
        run(exe, ["1500", p])
        f = oracle.read_ref_dump(p, 4, 32, 4, nf)["fields"]
        for k in range(4):
            assert np.array_equal(f[:, k], f[:, 1])
        extra = dict(T=f[4, 1], q=f[5:8, 1]) if nf == 8 else {}
        np.savez_compressed(os.path.join(OUT, name), rho=f[0, 1], u=f[1:4, 1], ny=30, Re=20.0, steps=1500, **extra)

    # staircase 2D bodies, 300 steps
    for name, _, exe, nx, ny, nb, wr, wc in STAIRCASE:
        p = os.path.join(tmp, name + ".bin")
        pt = os.path.join(tmp, name + ".types")
        run(exe, ["300", p, pt])
        r = oracle.read_ref_dump(p, nx + 2, ny + 2, 3, 4)
        fl = r["fields"][:3, 1]
        rest = np.fromfile(p)[4 * (nx + 2) * (ny + 2) * 3:].reshape(nb, 2, 300)
        types = np.fromfile(pt, dtype=np.uint8).reshape(ny + 2, nx + 2)
        np.savez_compressed(os.path.join(OUT, "staircase2d_%s_300.npz" % name), cl=rest[:, 0], cd=rest[:, 1],
                            types=types, window=fl[:, wr, wc], wrows=np.array([wr.start, wr.stop]),
                            wcols=np.array([wc.start, wc.stop]), sums=fl.reshape(3, -1).sum(axis=1), steps=300)
    triangle_details(tmp)
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
