"""Generate tests/golden/*.npz from the reference's own C core.

Runs src/Imaging/c/wem.c (+ shotwem.c, seismic.c) compiled UNMODIFIED in
oracle/_ref/ (see oracle/Makefile; FFTW 3.3.4 is replaced by oracle/fftw_subset.c)
on small seeded cases and stores inputs and outputs. Needs the reference sources,
so it runs in the build container only; the fixtures then pin the oracle and the
GPU path wherever the tests run.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "seismic.jl_gb300"))

import oracle as O  # noqa: E402
from wemgpu import seis, synth  # noqa: E402

CASES = {
    # name: (seed, nx, nz, nt, pspi, nref, fmax, padx, padt)
    "ss_64": (11, 64, 24, 128, 0, 2, 40.0, 2, 2),
    "ss_128_taper": (12, 128, 20, 128, 0, 2, 30.0, 2, 2),
    "pspi_64": (13, 64, 24, 128, 1, 4, 40.0, 2, 2),
    "pspi_128_r8": (14, 128, 16, 96, 1, 8, 30.0, 2, 1),
    "pspi_64_padx1": (15, 64, 12, 64, 1, 3, 40.0, 1, 2),
    # row lengths nkx = padx*nmx that are not powers of two (FFTW plans any length, wem.c:103-104)
    "pspi_500_padx2": (16, 500, 12, 256, 1, 4, 30.0, 2, 2),   # nkx 1000 = 2^3 5^3
    "ss_300_padx2": (17, 300, 12, 96, 0, 2, 30.0, 2, 2),      # nkx 600, taper on
    "pspi_768_padx2": (18, 768, 8, 64, 1, 3, 25.0, 2, 2),     # nkx 1536 = 2^9 3
    "pspi_97_padx1": (19, 97, 16, 96, 1, 4, 40.0, 1, 2),      # nkx 97, a prime
    "ss_50_padx1": (20, 50, 16, 96, 0, 2, 40.0, 1, 2),        # nkx 50
    # the source and the receivers below the surface (sz, gz in m; wem.c:213-224)
    "ss_64_buried": (23, 64, 24, 128, 0, 2, 40.0, 2, 2, 45.0, 95.0),
    "pspi_64_buried": (24, 64, 24, 128, 1, 4, 40.0, 2, 2, 95.0, 45.0),
    # padt = 1 with an odd trace length: f_op's transform is one sample shorter than the trace
    # (ntfft = 2 truncf(nt / 2)), so the last sample takes no part in migration; modelling
    # reads past the reference's buffer for that sample, so these pin migration only
    "pspi_64_nt97_padt1": (25, 64, 16, 97, 1, 4, 40.0, 2, 1),
    "ss_64_nt97_padt1": (26, 64, 16, 97, 0, 2, 40.0, 2, 1),
}


def case_inputs(seed, nx, nz, nt, pspi, nref, fmax, padx, padt, sz=0.0, gz=0.0):
    c = synth.small_case(seed, nx=nx, nz=nz, nt=nt, nshot=1, pspi=pspi, nref=nref, fmax=fmax, padx=padx,
                         padt=padt)
    p = dict(c["params"])
    p["sx"] = float(c["shots"].sx[0])
    if sz or gz:
        p["sz"], p["gz"] = float(sz), float(gz)
    d = synth.shot_gather_full(c["shots"], 0, nx)
    rng = np.random.default_rng(seed + 100)
    m_in = rng.standard_normal((nx, nz)).astype(np.float32)
    return p, c["vel"], c["wav"], d, m_in


def main(only=None):
    O.build()
    if O.build_ref() is None:
        sys.exit("reference sources not found: golden vectors come from the reference itself")
    os.environ.setdefault("OMP_NUM_THREADS", "4")
    for name, args in CASES.items():
        if only and name not in only:
            continue
        p, vel, wav, d, m_in = case_inputs(*args)
        m_ref = O.wem_ref(p, vel, wav, d=d, adj=True)
        d_ref = O.wem_ref(p, vel, wav, m=m_in, adj=False)
        np.savez_compressed(os.path.join(HERE, f"wem_{name}.npz"), vel=vel, wav=wav, d=d, m_in=m_in,
                            m_ref=m_ref, d_ref=d_ref,
                            params=np.array(repr({k: v for k, v in p.items()})))
        print(name, "image norm", float(np.linalg.norm(m_ref)), "data norm", float(np.linalg.norm(d_ref)))
    if only:
        return

    # 3-D (nmy > 1): rank-2 transforms over (nkx, nky), wem.c:100-104
    for name, (seed, pspi) in {"ss3d_32": (21, 0), "pspi3d_32": (22, 1)}.items():
        c = synth.small_case3d(seed, nx=32, ny=32, nz=8, nt=64, pspi=pspi, nref=3)
        p = dict(c["params"], sx=float(c["shots"].sx[0]), sy=float(c["shots"].sy[0]))
        d = c["shots"].data
        rng = np.random.default_rng(seed + 100)
        m_in = rng.standard_normal((32 * 32, 8)).astype(np.float32)
        m_ref = O.wem_ref(p, c["vel"], c["wav"], d=d, adj=True)
        d_ref = O.wem_ref(p, c["vel"], c["wav"], m=m_in, adj=False)
        np.savez_compressed(os.path.join(HERE, f"wem_{name}.npz"), vel=c["vel"], wav=c["wav"], d=d, m_in=m_in,
                            m_ref=m_ref, d_ref=d_ref, params=np.array(repr(p)))
        print(name, "image norm", float(np.linalg.norm(m_ref)))

    # file-level: the reference's main() on seis files (shotwem.c:12-140)
    p, vel, wav, d, _ = case_inputs(*CASES["pspi_64"])
    with tempfile.TemporaryDirectory() as td:
        seis.write_grid(os.path.join(td, "vel"), vel, o1=0.0, d1=p["dz"], ox=p["omx"], dx=p["dmx"])
        seis.write_wavelet(os.path.join(td, "wav"), wav, dt=p["dt"])
        seis.write_shot(os.path.join(td, "d"), d, sx=p["sx"], dt=p["dt"], ox=p["omx"], dx=p["dmx"])
        argv = [os.path.join(O.HERE, "_ref", "shotwem_ref"), "adj=y", "pspi=y", f"nref={p['nref']}",
                "d=" + os.path.join(td, "d"), "m=" + os.path.join(td, "m"), "vel=" + os.path.join(td, "vel"),
                "wav=" + os.path.join(td, "wav"), f"sx={p['sx']}", "sy=0", "sz=0", "gz=0",
                f"fmin={p['fmin']}", f"fmax={p['fmax']}", f"padt={p['padt']}", f"padx={p['padx']}", "verbose=n"]
        subprocess.run(argv, check=True, cwd=td)
        m_main, hdr, ext = seis.read(os.path.join(td, "m"))
        np.savez_compressed(os.path.join(HERE, "main_pspi_64.npz"), vel=vel, wav=wav, d=d, m_ref=m_main,
                            imx=np.array([h["imx"] for h in hdr]), mx=np.array([h["mx"] for h in hdr]),
                            n=np.array(ext["n"]), o=np.array(ext["o"]), dd=np.array(ext["d"]),
                            params=np.array(repr(p)))
        print("main() image norm", float(np.linalg.norm(m_main)))


EWEM_CASES = {
    # name: (seed, nx, nz, nt, fmax, padx[, sz, gz]); the S velocity is vp / 1.8 with a seeded
    # wobble; sz, gz (m) put the source and the receivers below the surface
    "ewem_64": (41, 64, 16, 128, 40.0, 2),        # nkx 128
    "ewem_150_padx1": (42, 150, 12, 128, 35.0, 1),  # nkx 150 (taper on)
    "ewem_64_buried": (43, 64, 16, 128, 40.0, 2, 35.0, 25.0),  # source from z = 40 m, receivers from 30 m
}


def ewem_main(only=None):
    """The reference's elastic ewem() (oracle/_ref/libewem_ref.so, src/Imaging/c/ewem.c),
    one shot per case, migration and forward; `only` limits it to the named cases."""
    os.environ.setdefault("OMP_NUM_THREADS", "4")
    for name, case in EWEM_CASES.items():
        if only and name not in only:
            continue
        seed, nx, nz, nt, fmax, padx = case[:6]
        sz, gz = case[6:8] if len(case) > 6 else (0.0, 0.0)
        c = synth.small_case(seed, nx=nx, nz=nz, nt=nt, nshot=1, pspi=0, fmax=fmax, padx=padx)
        rng = np.random.default_rng(seed + 200)
        vp = c["vel"]
        vs = (vp / 1.8 * (1.0 + 0.05 * rng.standard_normal(vp.shape))).astype(np.float32)
        p = dict(c["params"], sx=float(c["shots"].sx[0]), fmin=3.0, sz=sz, gz=gz)
        d = synth.shot_gather_full(c["shots"], 0, nx)
        ux_in = (0.4 * d + 0.1 * np.roll(d, 3, axis=1)).astype(np.float32)
        uz_in = d
        m_pp, m_s1, m_s2 = O.ewem_ref(p, vp, vs, c["wav"], ux=ux_in, uz=uz_in, adj=True)
        mpp_in = rng.standard_normal((nx, nz)).astype(np.float32)
        mps2_in = rng.standard_normal((nx, nz)).astype(np.float32)
        ux_ref, uy_ref, uz_ref = O.ewem_ref(p, vp, vs, c["wav"], mpp=mpp_in, mps2=mps2_in, adj=False)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), vp=vp, vs=vs, wav=c["wav"], ux=ux_in, uz=uz_in,
                            mpp_ref=m_pp, mps2_ref=m_s2, mpp_in=mpp_in, mps2_in=mps2_in, ux_ref=ux_ref,
                            uz_ref=uz_ref, params=np.array(repr(p)))
        print(name, "images", float(np.linalg.norm(m_pp)), float(np.linalg.norm(m_s2)), "data",
              float(np.linalg.norm(ux_ref)), float(np.linalg.norm(uz_ref)))


# 3-D grids (nmy > 1): (seed, nx, ny, nz, nt, fmax, padx[, sz, gz]); planes of padx*nx x padx*ny
EWEM3D_CASES = {
    "ewem3d_32": (51, 32, 32, 8, 64, 40.0, 2),                    # 64 x 64 planes
    "ewem3d_64x32_buried": (53, 64, 32, 6, 32, 35.0, 2, 15.0, 25.0),  # 128 x 64 planes, source and receivers below the surface
    "ewem3d_128x32_taper": (54, 128, 32, 4, 32, 30.0, 2),          # 256 x 64 planes, the taper on along x
}
# the x component fed to the migration: a mix of the z component and its time shift


def ewem3d_ux(uz):
    return (0.4 * uz + 0.1 * np.roll(uz, 3, axis=1)).astype(np.float32)


def ewem3d_main(only=None):
    """The reference's elastic ewem() on 3-D grids (rank-2 transforms over the x-y planes,
    ewem.c:84-96), one shot per case, migration and forward."""
    os.environ.setdefault("OMP_NUM_THREADS", "4")
    for name, case in EWEM3D_CASES.items():
        if only and name not in only:
            continue
        seed, nx, ny, nz, nt, fmax, padx = case[:7]
        sz, gz = case[7:9] if len(case) > 7 else (0.0, 0.0)
        c = synth.small_case3d(seed, nx=nx, ny=ny, nz=nz, nt=nt, nshot=1, pspi=0, fmax=fmax, padx=padx)
        rng = np.random.default_rng(seed + 200)
        vp = c["vel"]
        vs = (vp / 1.8 * (1.0 + 0.05 * rng.standard_normal(vp.shape))).astype(np.float32)
        p = dict(c["params"], sx=float(c["shots"].sx[0]), sy=float(c["shots"].sy[0]), fmin=3.0, sz=sz, gz=gz)
        d = synth.shot_gather_full(c["shots"], 0, nx * ny)
        uz_in = d
        m_pp, m_s1, m_s2 = O.ewem_ref(p, vp, vs, c["wav"], ux=ewem3d_ux(uz_in), uz=uz_in, adj=True)
        mpp_in = rng.standard_normal((nx * ny, nz)).astype(np.float32)
        mps2_in = rng.standard_normal((nx * ny, nz)).astype(np.float32)
        ux_ref, uy_ref, uz_ref = O.ewem_ref(p, vp, vs, c["wav"], mpp=mpp_in, mps2=mps2_in, adj=False)
        # ux is not stored: ewem3d_ux(uz) rebuilds it
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), vp=vp, vs=vs, wav=c["wav"], uz=uz_in,
                            mpp_ref=m_pp, mps2_ref=m_s2, mpp_in=mpp_in, mps2_in=mps2_in, ux_ref=ux_ref,
                            uz_ref=uz_ref, params=np.array(repr(p)))
        print(name, "images", float(np.linalg.norm(m_pp)), float(np.linalg.norm(m_s2)), "data",
              float(np.linalg.norm(ux_ref)), float(np.linalg.norm(uz_ref)))


ANGLE_CASES = {
    # name: (seed, nx, nz, nt, fmax); nx > 100 switches the reference's taper on
    "angles_64": (31, 64, 24, 64, 40.0),
    "angles_128": (32, 128, 16, 64, 30.0),
}


def angles_main():
    """compute_angles() of the reference (wem.c:566-684), one shot per case. Run in a
    process with OMP_NUM_THREADS=1: the reference's frequency loop adds into shared
    arrays from every thread without synchronisation."""
    for name, (seed, nx, nz, nt, fmax) in ANGLE_CASES.items():
        c = synth.small_case(seed, nx=nx, nz=nz, nt=nt, nshot=1, pspi=0, fmax=fmax)
        p = dict(c["params"], sx=float(c["shots"].sx[0]))
        ax, ay = O.angles_ref(p, c["vel"], c["wav"])
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), vel=c["vel"], wav=c["wav"], angx=ax, angy=ay,
                            params=np.array(repr(p)))
        print(name, "angx range", float(ax.min()), float(ax.max()), "angy max", float(np.abs(ay).max()))
    # 3-D: both lateral axes (rank-3 transforms over nkx, nky, nkz, wem.c:630-641)
    c = synth.small_case3d(35, nx=64, ny=64, nz=8, nt=64, nshot=1, pspi=0, fmax=30.0)
    p = dict(c["params"], sx=float(c["shots"].sx[0]), sy=float(c["shots"].sy[0]))
    ax, ay = O.angles_ref(p, c["vel"], c["wav"])
    np.savez_compressed(os.path.join(HERE, "angles3d_64.npz"), vel=c["vel"], wav=c["wav"], angx=ax, angy=ay,
                        params=np.array(repr(p)))
    print("angles3d_64 angx range", float(ax.min()), float(ax.max()), "angy range", float(ay.min()), float(ay.max()))


if __name__ == "__main__":
    if sys.argv[1:] == ["angles"]:
        angles_main()
    elif sys.argv[1:2] == ["ewem"]:
        # python tests/golden/make_golden.py ewem [name,name...]: the elastic cases (or those named)
        O.build()
        if O.build_ref() is None:
            sys.exit("reference sources not found")
        ewem_main(set(sys.argv[2].split(",")) if len(sys.argv) > 2 else None)
    elif sys.argv[1:2] == ["ewem3d"]:
        # python tests/golden/make_golden.py ewem3d [name,name...]: the 3-D elastic cases
        O.build()
        if O.build_ref() is None:
            sys.exit("reference sources not found")
        ewem3d_main(set(sys.argv[2].split(",")) if len(sys.argv) > 2 else None)
    elif sys.argv[1:2] == ["--only"]:
        # python tests/golden/make_golden.py --only name[,name...]: those 2-D cases only
        main(set(sys.argv[2].split(",")))
    else:
        main()
        subprocess.run([sys.executable, os.path.abspath(__file__), "angles"], check=True,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
        ewem_main()
        ewem3d_main()
