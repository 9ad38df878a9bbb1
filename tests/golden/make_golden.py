"""Generate the golden vectors in tests/golden/ from the reference's own code.

Runs only where the reference sources exist: it builds oracle/_ref/libastref.so
(oracle/make_ref.py, the reference's functions compiled for the host) and
records their outputs on seeded inputs:

  faces.npz      HLL, HLLC, HLLC_Aleksashov and exact-Godunov fluxes + dt on 1024 random
                 states and on hand-picked states that reach every wave
                 pattern of the exact solver (two shocks, shock-rarefaction,
                 two rarefactions, vacuum) and the uniform-state case of the
                 reference's `test` kernel (kernel.cu:3095-3107);
  step_tvd.npz   20 launches of Kernel_TVD (kernel.cu:2513) + funk_time on a
                 96x12 grid with a random state;
  step_mk_hll.npz, step_mk_hllca.npz, step_mk_god.npz
                 20 launches of add_MK (kernel.cu:2293), method 0 (HLL),
                 method 1 (HLLC_Aleksashov) and method 2 (exact Godunov), on
                 a 48x24 axisymmetric grid;
  inflow.npz     one launch of add2_bound (kernel.cu:1895-1925, p_H = 7,
                 inflow speed 1) on a random old and new state, 24x8;
  step_mk_neutral.npz
                 20 launches of add_MK method 0 (HLL) on the 48x24 grid with
                 a random neutral-coupling source nn2 (kernel.cu:2495-2496;
                 the reference's main passes zeros);
  step_add2_m0.npz, step_add2_m1.npz
                 20 launches of add2 (kernel.cu:1928) + funk_time, method 0
                 and method 1 (the time-dependent inflow density), on a
                 96x12 grid with a random state;
  faces_scalar.npz
                 the passive-scalar solvers' fluxes (mass, momentum, energy,
                 scalar) + dt on the face states of faces.npz with random
                 scalars: the Q channel of HLLC_2d_Korolkov_b_s
                 (Gas_Dinamic.cu:1604-1811, metod 2) and HLLCQ_Korolkov_2D
                 (Gas_Dinamic.cu:249-353);
  step_scalar_hllc.npz, step_scalar_hllcq.npz
                 20 steps carrying a passive scalar on a 48x24 axisymmetric
                 blast-like grid, every face evaluated by those reference
                 functions (the reference's steps carry no scalar: the step
                 loop and the update are the oracle's);
  writers.npz    the bytes of the files the reference's writers produce for a
                 random 24x12 state: print_file_mini (kernel.cu:3109-3173)
                 with every 2nd and every 3rd cell, and the end-of-run block of
                 main (kernel.cu:4109-4221: the .bin dump, the mini Tecplot
                 file with T and Zav, the axis line, the run summary).

The configurations that reproduce those kernels live in golden_configs.py so
the tests use exactly the same ones.  Usage:
python tests/golden/make_golden.py [writers | add2 | scalar]   (that fixture only)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, HERE)

import make_ref  # noqa: E402
import pyoracle as O  # noqa: E402
import golden_configs as G  # noqa: E402


def face_cases(rng):
    cases = []
    for _ in range(1024):
        sL = [rng.uniform(0.1, 5.0), rng.uniform(0.05, 20.0)]
        sR = [rng.uniform(0.1, 5.0), rng.uniform(0.05, 20.0)]
        uL = list(rng.uniform(-5.0, 5.0, 2))
        uR = list(rng.uniform(-5.0, 5.0, 2))
        cases.append(sL + uL + sR + uR)
    # exact-solver wave patterns, normal along +z
    cases += [
        [1.0, 1.0, 2.0, 0.0, 1.0, 1.0, -2.0, 0.0],        # two shocks (colliding)
        [4.0, 10.0, 3.0, 0.5, 1.0, 1.0, -1.0, -0.5],      # two shocks, unequal
        [1.0, 1.0, 0.0, 0.0, 0.125, 0.1, 0.0, 0.0],       # Sod: shock + rarefaction
        [1.0, 0.4, -2.0, 0.0, 1.0, 0.4, 2.0, 0.0],        # 123 problem: two rarefactions
        [1.0, 0.1, -10.0, 0.3, 1.0, 0.1, 10.0, -0.3],     # vacuum generation
        [1.0, 0.0666666, -1.0, 0.0, 1.0, 0.0666666, -1.0, 0.0],  # `test` kernel state
        [1.0, 10.0, 0.0, 0.0, 1.0, 0.1, 0.0, 0.0],        # blast interface
        [2.0, 3.0, 0.7, 0.2, 2.0, 3.0, 0.7, 0.2],         # identical states
    ]
    return np.array(cases)


def make_faces(rng):
    cfg = G.face_config()
    O.ref_set(cfg)
    X = face_cases(rng)
    normals = [(1.0, 0.0), (-1.0, 0.0), (0.0, 1.0), (0.0, -1.0)]
    n = np.array([normals[i % 4] for i in range(len(X))])
    n[-8:] = (1.0, 0.0)
    rad = np.where(n[:, 0] != 0, 0.01, 0.02)
    out = {}
    for name, which in (("hll", 0), ("hllc", 1), ("godunov", 2), ("hllca", 3)):
        F = np.zeros((len(X), 4))
        T = np.zeros(len(X))
        for i, row in enumerate(X):
            T[i], F[i] = O.ref_face(which, row[0:2], row[2:4], row[4:6], row[6:8], n[i, 0], n[i, 1], rad[i])
        out[name + "_flux"] = F
        out[name + "_dt"] = T
    np.savez_compressed(os.path.join(HERE, "faces.npz"), states=X, normals=n, rad=rad,
                        gamma=cfg.gamma, cfl=cfg.cfl, **out)


def make_step(fname, cfg, kernel, method, nsteps, rng):
    K = cfg.N * cfg.M
    s, u = G.random_state(K, rng)
    s1, u1, tdo, tt, st = O.ref_run(kernel, cfg, s, u, nsteps, method=method)
    np.savez_compressed(os.path.join(HERE, fname), s0=s, u0=u, s=s1, u=u1, T_do=tdo, TT=tt,
                        steps=st, nsteps=nsteps)


def make_inflow(rng):
    cfg = G.inflow_config()
    K = cfg.N * cfg.M
    s, u = G.random_state(K, rng)
    s2, u2 = G.random_state(K, rng)
    b2, c2 = O.ref_bound(cfg, s, u, s2, u2)
    np.savez_compressed(os.path.join(HERE, "inflow.npz"), s=s, u=u, s2=s2, u2=u2, s2_out=b2, u2_out=c2)


def make_neutral(rng):
    cfg = G.add_mk_config(0)
    K = cfg.N * cfg.M
    s, u = G.random_state(K, rng)
    nn2 = rng.uniform(-0.5, 0.5, (K, 3))
    s1, u1, tdo, tt, st = O.ref_run(O.REF_ADD_MK, cfg, s, u, 20, method=0, nn2=nn2)
    np.savez_compressed(os.path.join(HERE, "step_mk_neutral.npz"), s0=s, u0=u, nn2=nn2, s=s1, u=u1, T_do=tdo,
                        TT=tt, steps=st, nsteps=20)


def make_add2():
    rng = np.random.default_rng(1928)
    for method in (0, 1):
        make_step(f"step_add2_m{method}.npz", G.add2_config(), O.REF_ADD2, method, 20, rng)


def make_scalar(rng):
    cfg = G.face_config()
    O.ref_set(cfg)
    X = face_cases(rng)
    Q = rng.uniform(0.0, 3.0, (len(X), 2))
    normals = [(1.0, 0.0), (-1.0, 0.0), (0.0, 1.0), (0.0, -1.0)]
    n = np.array([normals[i % 4] for i in range(len(X))])
    rad = np.where(n[:, 0] != 0, 0.01, 0.02)
    out = {}
    for name, which in (("hllc", 1), ("hllcq", 5)):
        F = np.zeros((len(X), 5))
        T = np.zeros(len(X))
        for i, row in enumerate(X):
            T[i], F[i] = O.ref_face_q(which, row[0:2], row[2:4], row[4:6], row[6:8], Q[i, 0], Q[i, 1], n[i, 0],
                                      n[i, 1], rad[i])
        out[name + "_flux"] = F
        out[name + "_dt"] = T
    np.savez_compressed(os.path.join(HERE, "faces_scalar.npz"), states=X, scalars=Q, normals=n, rad=rad,
                        gamma=cfg.gamma, cfl=cfg.cfl, **out)
    for name, flux in (("hllc", 1), ("hllcq", 4)):
        cfg = G.scalar_config(flux)
        K = cfg.N * cfg.M
        s, u = G.random_state(K, rng)
        q = s[:, 0] * rng.uniform(0.5, 1.5, K)
        s1, u1, q1, tdo, tt, st = O.run_scalar(cfg, s, u, q, 20, use_ref=True)
        np.savez_compressed(os.path.join(HERE, f"step_scalar_{name}.npz"), s0=s, u0=u, q0=q, s=s1, u=u1, q=q1,
                            T_do=tdo, TT=tt, steps=st, nsteps=20)


def make_writers(rng):
    import tempfile
    cfg = G.writer_config()
    K = cfg.N * cfg.M
    s, u = G.random_state(K, rng)
    u[:, 0] -= 0.5
    TT, mach_inf, chi, soltime = 0.0123456789, 0.5, 17.0, 0.25
    files = {}
    with tempfile.TemporaryDirectory() as d:
        for stride in (2, 3):
            p = os.path.join(d, f"pfm{stride}.txt")
            O.ref_print_file_mini(cfg, s, u, stride, soltime, p)
            files[f"pfm{stride}"] = open(p, "rb").read()
            name = os.path.join(d, f"run{stride}")
            O.ref_end_of_run(cfg, s, u, TT, stride, mach_inf, chi, name)
            files[f"final{stride}"] = open(name + "_param_for_texplot_mini.txt", "rb").read()
            if stride == 2:
                files["bin"] = open(name + ".bin", "rb").read()
                files["axis"] = open(name + "_param_y=0.txt", "rb").read()
                files["inform"] = open(name + "_inform.txt", "rb").read()
    np.savez_compressed(os.path.join(HERE, "writers.npz"), s=s, u=u, TT=TT, mach_inf=mach_inf, chi=chi,
                        soltime=soltime, **{k: np.frombuffer(v, dtype=np.uint8) for k, v in files.items()})


def main():
    make_ref.main([])
    if sys.argv[1:] == ["writers"]:
        make_writers(np.random.default_rng(3109))
        print("writers.npz written to", HERE)
        return
    if sys.argv[1:] == ["add2"]:
        make_add2()
        print("add2 fixtures written to", HERE)
        return
    if sys.argv[1:] == ["scalar"]:
        make_scalar(np.random.default_rng(249))
        print("scalar fixtures written to", HERE)
        return
    rng = np.random.default_rng(20261203)
    make_faces(rng)
    make_step("step_tvd.npz", G.tvd_config(), O.REF_KERNEL_TVD, 1, 20, rng)
    make_step("step_mk_hll.npz", G.add_mk_config(0), O.REF_ADD_MK, 0, 20, rng)
    make_step("step_mk_god.npz", G.add_mk_config(2), O.REF_ADD_MK, 2, 20, rng)
    make_step("step_mk_hllca.npz", G.add_mk_config(1), O.REF_ADD_MK, 1, 20, rng)
    make_inflow(np.random.default_rng(1895))
    make_neutral(np.random.default_rng(2495))
    make_writers(np.random.default_rng(3109))
    make_add2()
    make_scalar(np.random.default_rng(249))
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
