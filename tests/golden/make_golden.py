"""Generate the golden fixtures in this directory from the FP64 oracle.

    python tests/golden/make_golden.py

The oracle (oracle/, a C restatement of Sunny.jl's algorithm for this path) runs on
seeded inputs of small models; inputs and outputs are stored in oracle_small.npz. The
CPU tests check that the oracle built on the current machine reproduces them (the
oracle is compiled on every machine that runs the tests, x86 here and Arm on the GPU
host), and the GPU tests check the CUDA path against the same numbers.

Julia is not available, so these are oracle outputs, not outputs of Sunny itself; the
oracle is pinned separately against the reference tests' known answers
(test_oracle_known_answers.py).
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import __graft_entry__ as ge  # noqa: E402
from models import rich_dipole, rich_sun  # noqa: E402

OUT = HERE / "oracle_small.npz"


def diamond_sqw_model(sg):
    """test_correlation_sampling.jl:156-169: diamond 2x3x4, s=3/2, J=0.6498 on Bond(1,3,[0,0,0])."""
    sys_ = sg.System(sg.diamond_crystal(), [(1, sg.Moment(s=1.5, g=2))], "dipole", dims=(2, 3, 4), seed=101,
                     device=None)
    sys_.set_exchange(0.6498, sg.Bond(1, 3, [0, 0, 0]))
    sys_.randomize_spins()
    return sys_


def sqw_params(sg, sys_):
    """Sampler parameters of SampledCorrelations(sys; energies=range(0, 5.5, 10), dt=0.12,
    measure=ssf_perp(sys)) (SampledCorrelations.jl:152-173, 199-269)."""
    energies = np.linspace(0.0, 5.5, 10)
    dt, measperiod = sg.adjusted_dt_and_downsampling_factor(0.12, len(energies), energies[-1])
    m = sg.ssf_perp(sys_)
    return dict(dt=dt, measperiod=measperiod, n_all_omega=2 * (len(energies) - 1), obs=m.observables,
                pairs=m.corr_pairs, nobs=m.nobs)


def generate():
    sg = ge.package()
    orc = ge.oracle()
    orc.load()
    out = {}
    rng = np.random.default_rng(20261203)

    # dipole mode, every coupling type: gradient, energy, Heun with injected noise, midpoint
    d = rich_dipole(sg, device=None)
    od = orc.OracleSystem.from_system(d)
    S0 = d.dipoles_flat()
    noise = rng.standard_normal((3, d.nsites, 3))
    out["dip_S0"] = S0
    out["dip_grad"] = od.grad(S0)
    out["dip_E"] = np.array(od.energy(S0))
    out["dip_noise"] = noise
    out["dip_heun3"], _ = od.langevin(S0, None, 0.01, 0.1, 0.3, 3, noise)
    st, Sm, _, it = od.midpoint(S0, None, 0.02, 0.0, 1e-12, 100, 3)
    assert st == 0
    out["dip_mid3"] = Sm

    # SU(3) with biquadratic couplings
    s = rich_sun(sg, N=3, device=None)
    os_ = orc.OracleSystem.from_system(s)
    Z0 = s.coherents_flat()
    zn = (rng.standard_normal((2, s.nsites, 3)) + 1j * rng.standard_normal((2, s.nsites, 3))) / np.sqrt(2)
    out["sun_Z0"] = Z0
    out["sun_grad"] = os_.grad(None, Z0)
    out["sun_E"] = np.array(os_.energy(s.dipoles_flat(), Z0))
    out["sun_noise"] = zn
    _, out["sun_heun2"] = os_.langevin(s.dipoles_flat(), Z0, 0.01, 0.1, 0.3, 2, zn)
    st, _, Zm, _ = os_.midpoint(s.dipoles_flat(), Z0, 0.02, 0.0, 1e-12, 100, 2)
    assert st == 0
    out["sun_mid2"] = Zm

    # one S(q,w) sample of the reference's golden configuration, from a seeded state
    q = diamond_sqw_model(sg)
    oq = orc.OracleSystem.from_system(q)
    p = sqw_params(sg, q)
    oc = orc.OracleCorrelations(oq, p["obs"].reshape(-1), p["nobs"], p["pairs"], p["n_all_omega"], p["measperiod"],
                                p["dt"], 1e-12)
    Sq0 = q.dipoles_flat()
    Sq1, _ = oc.add_sample(Sq0, None)
    data = oc.data                                   # [c, i, j, q1, q2, q3, w]
    out["sqw_S0"] = Sq0
    out["sqw_S1"] = Sq1
    out["sqw_sum_ij"] = data.sum(axis=(1, 2))        # [c, q1, q2, q3, w]
    out["sqw_block_00"] = data[:, 0, 0]              # [c, q1, q2, q3, w]
    out["sqw_block_37"] = data[:, 3, 7]

    # replica exchange on a 6-slot ladder with fixed uniforms (ParallelTempering.jl:40-73)
    E = rng.normal(-10.0, 2.0, 6)
    kT = np.geomspace(0.2, 1.5, 6)
    u = rng.random(6)
    for start in (1, 2):
        ids, acc = orc.replica_exchange(E, kT, list(range(6)), start, u)
        out[f"pt_ids_start{start}"] = np.asarray(ids)
        out[f"pt_acc_start{start}"] = np.asarray(acc)
    out["pt_E"], out["pt_kT"], out["pt_u"] = E, kT, u
    return out


if __name__ == "__main__":
    data = generate()
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(data)} arrays)")
