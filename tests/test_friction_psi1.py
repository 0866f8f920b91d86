"""The ensemble kernel's friction takes ψ2 = σ ψ1 / hypot(1, v ψ1) (equation.jl:237-244) as
σ / sqrt(v² + ψ1⁻²) with ψ1⁻¹ = exp(-(c1 + (b/a) ln θ)) from FP32 exp and log. Checked on the
states of an FP64 oracle run through earthquake cycles (the 80-km strike-slip fault over 50 years,
VCABM5, every 10th step): ψ1⁻¹ stays far below the slip rate, and the mixed form equals the
reference formula to FP64 rounding (the same as the reformulation carried out in FP64)."""
import numpy as np

from oetqf_gb300.workloads import YEAR, strike_slip_fault


def test_psi1_inverse_in_fp32_leaves_psi2_at_fp64_rounding(oracle):
    cm = strike_slip_fault(years=50.0)
    om = oracle.OracleModel(oracle.gf_ff(cm.mf, cm.lam, cm.mu), cm.pf)
    pf = cm.pf
    flat = lambda q: np.asarray(q, dtype=np.float64).reshape(-1, order="F")
    a, b, L, sig = flat(pf.a), flat(pf.b), flat(pf.L), flat(pf.σ)
    c1 = pf.f0 / a + (b / a) * np.log(pf.v0 / L) - np.log(2 * pf.v0)
    boa = b / a
    N = a.size
    _, st, t_rec, u_rec = oracle.integrate_record(om, cm.u0, 0.0, cm.horizon, stride=10, max_records=20000,
                                                  reltol=1e-6, abstol=1e-8, dt0=1e-8, dtmax=0.2 * YEAR, alg="VCABM5")
    assert st.status == 0 and t_rec.size > 100
    v, th = u_rec[:, :N], u_rec[:, N:2 * N]
    assert np.abs(v).max() > 1e-3  # the run passes through earthquakes (slip rates of cm/s)
    psi1 = np.exp(c1 + boa * np.log(th))
    assert (1.0 / psi1 / np.abs(v)).max() < 1e-6
    ref = sig * psi1 / np.hypot(1.0, v * psi1)
    e32 = np.exp(-(boa.astype(np.float32) * np.log(th.astype(np.float32)) + c1.astype(np.float32)))
    mixed = sig / np.sqrt(v * v + e32.astype(np.float64) ** 2)
    assert (np.abs(mixed - ref) / np.abs(ref)).max() < 1e-15
