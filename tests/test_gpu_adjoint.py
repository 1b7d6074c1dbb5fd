"""The discrete adjoint of the midpoint trajectory and S(q,ω) loss (GPU, FP64) against
central finite differences of the GPU loss, and against central finite differences of
the FP64 oracle (the CPU reference gradient), with h = 1e-4 as the differentiation
workload states."""
import numpy as np
import pytest

from adjoint_models import sc_params, sc_system, tangent

pytestmark = pytest.mark.gpu

THETA0 = np.array([1.0, 0.1, 0.05])
THETA_T = np.array([1.1, 0.08, 0.07])
H = 1e-4


def make_adjoint(sg, sys_, nw=6, wmax=16.0):
    return sg.SampledCorrelationsAdjoint(sys_, sc_params(sg), measure=sg.ssf_trace(sys_),
                                         energies=np.linspace(0.0, wmax, nw), dt=0.025)


def fd_grad(loss_at, theta, h=H):
    g = np.zeros(len(theta))
    for k in range(len(theta)):
        e = np.zeros(len(theta))
        e[k] = h
        g[k] = (loss_at(theta + e) - loss_at(theta - e)) / (2 * h)
    return g


def test_adjoint_matches_finite_differences(gpu, sg):
    sys_ = sc_system(sg, 4, THETA0)
    adj = make_adjoint(sg, sys_)
    assert adj.measperiod == 8 and adj.nsteps == 40
    S0 = sys_.dipoles_flat()
    adj.set_params(THETA_T)
    _, target = adj.loss(S0, return_data=True)
    adj.set_target(target)
    assert adj.loss(S0) == 0.0
    adj.set_params(THETA0)
    L, g = adj.loss_and_grad(S0, checkpoint=16)
    assert L > 0
    assert L == pytest.approx(adj.loss(S0), rel=1e-13)

    def loss_at(th):
        adj.set_params(th)
        return adj.loss(S0)

    fd = fd_grad(loss_at, THETA0)
    assert np.linalg.norm(g - fd) <= 1e-4 * np.linalg.norm(fd), (g, fd)
    # the checkpoint interval changes memory, not the result
    adj.set_params(THETA0)
    _, g8 = adj.loss_and_grad(S0, checkpoint=8)
    _, g40 = adj.loss_and_grad(S0, checkpoint=40)
    assert np.max(np.abs(g8 - g)) <= 1e-12 * np.max(np.abs(g))
    assert np.max(np.abs(g40 - g)) <= 1e-12 * np.max(np.abs(g))
    adj.close()


def test_adjoint_state_gradient(gpu, sg):
    sys_ = sc_system(sg, 4, THETA0, seed=11)
    adj = make_adjoint(sg, sys_)
    S0 = sys_.dipoles_flat()
    adj.set_params(THETA_T)
    _, target = adj.loss(S0, return_data=True)
    adj.set_target(target)
    adj.set_params(THETA0)
    _, _, gS = adj.loss_and_grad(S0, checkpoint=16, state_grad=True)
    d = tangent(S0, np.random.default_rng(1))
    eps = 1e-5
    fd = (adj.loss(S0 + eps * d) - adj.loss(S0 - eps * d)) / (2 * eps)
    assert np.sum(gS * d) == pytest.approx(fd, rel=1e-4)
    adj.close()


def test_adjoint_matches_oracle_reference_gradient(gpu, sg, orc):
    # FP64 CPU reference on a 6x6x6 copy: central differences of the oracle's loss
    from sunny_gb300.adjoint import twin_system
    sys_ = sc_system(sg, 6, THETA0, seed=7)
    adj = make_adjoint(sg, sys_)
    S0 = sys_.dipoles_flat()
    m = sg.ssf_trace(sys_)
    obs = np.ascontiguousarray(m.observables, dtype=float).reshape(-1)

    def oracle_loss(theta, target):
        twin = twin_system(sys_)
        for f, v in zip(sc_params(sg), theta):
            f(twin, float(v))
        o = orc.OracleSystem.from_system(twin)
        return orc.sqw_loss(o, obs, m.nobs, m.corr_pairs, adj.n_all_omega, adj.measperiod, adj.dt, 1e-12, S0, target)

    zero = np.zeros(adj.shape, dtype=complex)
    _, target = oracle_loss(THETA_T, zero)
    adj.set_target(target)
    fd = fd_grad(lambda th: oracle_loss(th, target)[0], THETA0)
    adj.set_params(THETA0)
    L, g = adj.loss_and_grad(S0, checkpoint=16)
    assert L == pytest.approx(oracle_loss(THETA0, target)[0], rel=1e-9)
    assert np.linalg.norm(g - fd) <= 1e-4 * np.linalg.norm(fd), (g, fd)
    adj.close()


def test_adjoint_rejects_unsupported_couplings(gpu, sg):
    sys_ = sc_system(sg, 4, THETA0)
    sys_.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]), biquad=0.1)
    with pytest.raises(sg.SunnyGPUError, match="bilinear"):
        make_adjoint(sg, sys_)
