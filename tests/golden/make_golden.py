"""Writes the golden fixtures in tests/golden/ from the reference's own code.

Run in a checkout where the reference sources are available:
    sh oracle/build_ref.sh /path/to/gasoline && python tests/golden/make_golden.py
It calls the reference's pkdBuildBinary/pkdGravAll and smSmooth/smReSmooth
through oracle/_ref/libgasref.so on small seeded inputs and stores inputs
and outputs as compressed .npz files.  The tests compare the CPU oracle and
the CUDA path against these files, so they need no reference at run time.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..")))
import oracle  # noqa: E402
from gasoline_gb300 import ics  # noqa: E402
from golden_io import render_frames  # noqa: E402


def grav_case(name, pos, mass, soft, gp):
    R = oracle.reference()
    g = R.grav(pos, mass, soft, gp)
    inode, dnode, perm = R.tree(pos, mass, soft, gp)
    bl = R.lists(pos, mass, soft, gp)
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"), pos=pos, mass=mass, soft=soft,
        params=np.array([gp.nBucket, gp.iOrder, gp.bPeriodic, gp.bEwald,
                         gp.iEwOrder, gp.nReps, gp.dTheta, gp.dPeriod,
                         gp.fEwCut, gp.fEwhCut]),
        acc=g["acc"], pot=g["pot"], dtGrav=g["dtGrav"], counters=g["counters"],
        inode=inode, dnode=dnode, perm=perm, blist=bl)
    print(name, len(mass), "nodes", len(inode), "buckets", len(bl))


def sph_case(name, pos, vel, mass, soft, u, sp):
    R = oracle.reference()
    r = R.sph(pos, vel, mass, soft, u, sp)
    out = np.stack([r[k] for k in oracle.SPH_FIELDS], axis=1)
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"), pos=pos, vel=vel, mass=mass,
        soft=soft, u=u,
        params=np.array([sp.nSmooth, sp.bPeriodic, sp.dPeriod, sp.alpha,
                         sp.beta, sp.gamma, sp.dEtaCourant, sp.nBucket,
                         sp.iViscosityLimiter]),
        out=out, dtNew=r["dtNew"], mumax=r["mumax"])
    print(name, len(mass))


def high_order_cases():
    """Octopole and hexadecapole cells (iOrder 3 and 4, the reference's
    default order): a Plummer sphere and a periodic lattice box."""
    pos, vel, m = ics.plummer(2048, seed=24)
    grav_case("grav_plummer_2k_o4", pos, m, np.full(len(m), 0.01),
              oracle.grav_params(periodic=False, iOrder=4))
    grav_case("grav_plummer_2k_o3", pos, m, np.full(len(m), 0.01),
              oracle.grav_params(periodic=False, iOrder=3))
    pos, vel, m = ics.lattice_box(8, seed=25)
    grav_case("grav_box_8_o4", pos, m, np.full(len(m), 1.0 / (50 * 8)),
              oracle.grav_params(periodic=True, ewald=True, iOrder=4))


def sph_box_case():
    """Periodic SPH: a 16^3 gas lattice in the unit box displaced by a
    Gaussian random field (rms 0.25 of the spacing), velocities from the
    displacements plus noise, u spread over [0.05, 0.15]; nSmooth 32, so
    most balls reach through a face of the box.  Besides ref_sph's fields
    the reference's own kNN sets are stored (ref_knn_sets: nnList size and
    member hash per particle)."""
    pos, vel, m = ics.lattice_box(16, seed=34, rms_frac=0.25)
    n = len(m)
    rng = np.random.default_rng(35)
    vel = vel * 50.0 + rng.normal(0.0, 0.05, (n, 3))
    u = rng.uniform(0.05, 0.15, n)
    soft = np.full(n, 0.001)
    sp = oracle.sph_params(nSmooth=32, periodic=True, L=1.0)
    sph_case("sph_box_16", pos, vel, m, soft, u, sp)
    k = oracle.reference_knn_sets(pos, m, soft, sp)
    d = dict(np.load(os.path.join(HERE, "sph_box_16.npz")))
    np.savez_compressed(os.path.join(HERE, "sph_box_16.npz"), **d, knn_hash=k["nbr_hash"],
                        knn_count=k["nbr_count"])


def particle_layout():
    """The reference's PARTICLE layout (sizeof and field offsets of this
    build, -DGASOLINE -DNOCOOLING) for the GPU tests of the store entry
    points, which run where the reference's headers are absent."""
    import json
    lay = oracle.reference_particle_layout()
    with open(os.path.join(HERE, "particle_layout.json"), "w") as f:
        json.dump(lay, f, indent=1, sort_keys=True)
        f.write("\n")
    print("particle layout", lay["stride"], "bytes")


def tipsy_fields(ng, nd, ns, seed):
    """Seeded particles of every Tipsy type; a few values sit on float
    rounding edges (subnormal, -0.0, near FLT_MAX, halfway between floats)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = ng + nd + ns
    pos = rng.normal(0.0, 1.0, (n, 3))
    vel = rng.normal(0.0, 1.0, (n, 3))
    f = np.zeros((n, 9))
    f[:, 0] = rng.uniform(0.1, 1.0, n)
    f[:, 1] = rng.uniform(0.01, 0.02, n)
    f[:ng, 2] = rng.uniform(1.0, 2.0, ng)
    f[:ng, 3] = rng.uniform(0.0, 5.0, ng)
    f[:ng, 4] = rng.uniform(0.0, 0.02, ng)
    f[ng + nd:, 4] = rng.uniform(0.0, 0.02, ns)
    f[ng + nd:, 5] = rng.uniform(0.0, 1.0, ns)
    f[:, 6] = rng.normal(-1.0, 0.1, n)
    pos[0] = [1e-40, -0.0, 3.0e38]
    pos[1] = [1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -24, -(1.0 + 2.0 ** -24)]
    vel[2] = [1e-45, -1e-39, 0.1]
    return pos, vel, f


def tipsy_case(name, ng, nd, ns, seed, dvFac=1.3, duTFac=2.5, rvFac=0.7, rTuFac=0.4):
    """A snapshot written by the reference's pkdWriteTipsy in both forms,
    and what its pkdReadTipsy reads back (with other unit factors)."""
    pos, vel, f = tipsy_fields(ng, nd, ns, seed)
    out = {}
    for std, tag in ((1, "std"), (0, "nat")):
        path = os.path.join(HERE, f"{name}.{tag}")
        oracle.reference_tipsy_write(path, std, 0.25, ng, nd, ns, pos, vel, f,
                                     dvFac=dvFac, duTFac=duTFac)
        p, v, q = oracle.reference_tipsy_read(path, std, ng, nd, ns, dvFac=rvFac, dTuFac=rTuFac)
        out[f"pos_{tag}"], out[f"vel_{tag}"], out[f"f_{tag}"] = p, v, q
    np.savez_compressed(os.path.join(HERE, name + ".npz"), pos=pos, vel=vel, f=f,
                        counts=np.array([ng, nd, ns]),
                        factors=np.array([dvFac, duTFac, rvFac, rTuFac]), time=0.25, **out)
    print(name, ng, nd, ns)


def multistep_cases():
    """Adaptive timesteps: force passes over an active subset, and a whole
    run of msrTopStepKDK with rungs, from the reference's own code."""
    rng = np.random.Generator(np.random.PCG64(17))
    pos, vel, m = ics.plummer(3000, seed=18)
    soft = np.full(len(m), 0.01)
    rung = rng.integers(0, 3, len(m)).astype(np.int32)
    gp = oracle.grav_params(periodic=False)
    g = oracle.reference_grav_active(pos, m, soft, rung, 1, gp)
    np.savez_compressed(os.path.join(HERE, "ms_active_grav.npz"), pos=pos, mass=m, soft=soft,
                        rung=rung, iRung=1, acc=g["acc"], pot=g["pot"], dtGrav=g["dtGrav"],
                        counters=g["counters"])
    pos, vel, m, u = ics.gas_sphere(3000, seed=19)
    vel = rng.normal(0.0, 0.2, pos.shape)
    soft = np.full(len(m), 0.01)
    rung = rng.integers(0, 3, len(m)).astype(np.int32)
    sp = oracle.sph_params(nSmooth=32)
    keys = ("acc", "uDotPdV", "uDotAV", "dtNew", "mumax", "dt", "fDensity")
    out = {}
    for iRung in (1, 2):   # two thirds and one third of the gas active
        s = oracle.reference_sph_active(pos, vel, m, soft, u, rung, iRung, sp)
        out.update({f"{k}_r{iRung}": s[k] for k in keys})
    np.savez_compressed(os.path.join(HERE, "ms_active_sph.npz"), pos=pos, vel=vel, mass=m,
                        soft=soft, u=u, rung=rung, **out)
    pg, vg, mg, ug = ics.gas_sphere(2000, seed=20)
    pd, vd, md = ics.plummer(1000, seed=21)
    pos = np.concatenate([pg, pd]); vel = np.concatenate([vg, vd])
    m = np.concatenate([0.2 * mg, 0.8 * md]); soft = np.full(len(m), 0.02)
    st = oracle.step_params(nSteps=3, iMaxRung=5, dDelta=0.05)
    r = oracle.reference_multistep(pos, vel, m, soft, 2000, ug, gp, sp, st)
    np.savez_compressed(os.path.join(HERE, "ms_run.npz"), pos0=pos, vel0=vel, mass=m, soft=soft,
                        u0=ug, ngas=2000, steps=np.array([st.nSteps, st.iMaxRung]),
                        dDelta=st.dDelta, **{k: np.asarray(v) for k, v in r.items()})
    print("multistep cases: run max rungs", r["maxRung"], "force passes", r["counts"])


def render_case():
    """TSC frames of gas, dark matter and stars through the reference's
    dfRenderParticles, gas balls and densities from the reference's SPH."""
    pg, vg, mg, ug = ics.gas_sphere(2000, seed=22)
    pd, vd, md = ics.plummer(1000, seed=23)
    pos = np.concatenate([pg, pd]); n = len(pos)
    mass = np.concatenate([0.2 * mg, 0.8 * md]); soft = np.full(n, 0.02)
    sph = oracle.reference().sph(pg, vg, mg * 0.2, soft[:2000], ug, oracle.sph_params(nSmooth=32))
    fb = np.concatenate([sph["fBall2"], np.zeros(n - 2000)])
    rho = np.concatenate([sph["fDensity"], np.zeros(n - 2000)])
    out = {}
    for k, rp in enumerate(render_frames()):
        out[f"img{k}"] = oracle.reference_render_tsc(pos, mass, soft, fb, rho, 2000, 100, rp)
    np.savez_compressed(os.path.join(HERE, "render_tsc.npz"), pos=pos, mass=mass, soft=soft,
                        u=ug, ngas=2000, nstar=100, fBall2=fb, fDensity=rho, **out)
    print("render frames", [float(out[k].sum()) for k in sorted(out)])


def main():
    if not oracle.reference_available():
        oracle.build_reference()
    pos, vel, m = ics.plummer(2048, seed=11)
    grav_case("grav_plummer_2k", pos, m, np.full(len(m), 0.01),
              oracle.grav_params(periodic=False))
    pos, vel, m = ics.lattice_box(8, seed=12)
    grav_case("grav_box_8", pos, m, np.full(len(m), 1.0 / (50 * 8)),
              oracle.grav_params(periodic=True, ewald=True))
    pos, vel, m = ics.uniform_cube(1500, seed=13)
    grav_case("grav_cube_soft", pos, m, np.full(len(m), 0.15),
              oracle.grav_params(periodic=False, nBucket=8, theta=0.7))
    high_order_cases()
    pos, vel, m, u = ics.gas_sphere(2048, seed=14)
    rng = np.random.Generator(np.random.PCG64(15))
    vel = rng.normal(0.0, 0.1, (len(m), 3))
    sph_case("sph_sphere_2k", pos, vel, m, np.full(len(m), 0.01), u,
             oracle.sph_params(nSmooth=32))
    sph_box_case()
    particle_layout()
    tipsy_case("tipsy_mixed", 300, 500, 200, seed=16)
    multistep_cases()
    render_case()


if __name__ == "__main__":
    # one group of fixtures only:
    #   python make_golden.py tipsy|multistep|render|sph_box|layout|high_order
    if len(sys.argv) > 1 and sys.argv[1] in ("tipsy", "multistep", "render", "sph_box", "layout",
                                             "high_order"):
        if not oracle.reference_available():
            oracle.build_reference()
        if sys.argv[1] == "tipsy":
            tipsy_case("tipsy_mixed", 300, 500, 200, seed=16)
        elif sys.argv[1] == "multistep":
            multistep_cases()
        elif sys.argv[1] == "sph_box":
            sph_box_case()
        elif sys.argv[1] == "layout":
            particle_layout()
        elif sys.argv[1] == "high_order":
            high_order_cases()
        else:
            render_case()
    else:
        main()
