"""gbc_rhs_visco_noalloc: the viscoelastic right-hand side for callers that cannot allocate device
memory when they evaluate it (code running while another library captures the CUDA stream, hosts
whose device memory belongs to their own pool, raw-pointer bindings). Every buffer is the
caller's; the library's only scratch is a fixed device array. Its results must equal the regular
entry point's. This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from oetqf_gb300 import PowerLawViscosityProperty, RateStateQuasiDynamicProperty, gen_hex8_box, gen_mesh

RTOL = 1e-6


def _model(oracle):
    mf = gen_mesh("RectOkada", 100.0, 100.0, 10.0, 20.0, 90.0)
    ma = gen_hex8_box(-100.0, -50.0, -20.0, 200.0, 100.0, -30.0, 2, 3, 4)
    lam = mu = 1.0
    st = oracle.gf_ff(mf, lam, mu)
    g12, g21, g22 = oracle.gf_fm(mf, ma, lam, mu), oracle.gf_mf(ma, mf, lam, mu), oracle.gf_mm(ma, lam, mu)
    rng = np.random.default_rng(21)
    pf = RateStateQuasiDynamicProperty(*[rng.random((mf.nx, mf.nξ)) for _ in range(4)], *rng.random(4))
    pa = PowerLawViscosityProperty(rng.random(ma.ne), 3 * np.ones(ma.ne), rng.random(6))
    return mf, ma, st, g12, g21, g22, pf, pa


def test_rejects_models_beyond_the_fixed_scratch():
    from oetqf_gb300 import _capi as C
    deps0 = np.zeros(6)
    fake = ctypes.c_void_p(16)
    # npad + 6 ne = 32 + 6 * 200000 > 1048576: refused before any device work
    rc = C.lib().gbc_rhs_visco_noalloc(4, 8, 200000, fake, fake, 1300000, fake, 1200000, fake, fake, fake, fake,
                                      1.0, 1.0, 0.6, 1e-6, fake, fake, C.ptr(deps0), fake, fake, None)
    assert rc == -1
    assert "fixed scratch" in C.last_error()


def test_rejects_misaligned_green_function_rows():
    """gm and g21 are read as 16-byte pairs; a view starting 8 bytes into a buffer is refused on
    the host, before any device work (the pointers are never dereferenced)."""
    from oetqf_gb300 import _capi as C
    deps0 = np.zeros(6)
    ok, off = ctypes.c_void_p(256), ctypes.c_void_p(256 + 8)
    N, ne = 32, 4
    for gm, g21 in ((off, ok), (ok, off)):
        rc = C.lib().gbc_rhs_visco_noalloc(4, 8, ne, ok, gm, N + 6 * ne, g21, 6 * ne, ok, ok, ok, ok,
                                          1.0, 1.0, 0.6, 1e-6, ok, ok, C.ptr(deps0), ok, ok, None)
        assert rc == -1
        assert "16-byte aligned" in C.last_error()


@pytest.mark.gpu
def test_noalloc_matches_regular_rhs_twice(oracle):
    torch = pytest.importorskip("torch")
    from oetqf_gb300 import _capi as C
    from oetqf_gb300.equation import GB300Model
    mf, ma, st, g12, g21, g22, pf, pa = _model(oracle)
    N, ne = mf.nx * mf.nξ, ma.ne
    M = 6 * ne
    # regular entry point
    m = GB300Model(mf.nx, mf.nξ, ne)
    m.set_gf(C.GBC_GF11_REAL, st)
    m.set_gf(C.GBC_GF12, g12)
    m.set_gf(C.GBC_GF21, g21)
    m.set_gf(C.GBC_GF22, g22)
    m.set_fault_props(pf)
    m.set_mantle_props(pa)
    # caller-owned device buffers in the documented layouts
    dev = lambda a: torch.tensor(np.ascontiguousarray(a, dtype=np.float64).reshape(-1), device="cuda:0")
    npad = (N + 31) // 32 * 32
    ldm = npad + M
    gm = np.zeros((M, ldm))
    gm[:, :N], gm[:, npad:npad + M] = g12, g22
    d_st, d_gm, d_g21 = dev(st.reshape(-1, order="F")), dev(gm), dev(g21)
    d_a, d_b, d_L, d_s = (dev(q.reshape(-1, order="F")) for q in (pf.a, pf.b, pf.L, pf.σ))
    d_gam, d_n = dev(pa.γ), dev(pa.n)
    deps0 = np.ascontiguousarray(pa.dϵ0)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(22)
    free_after_first = None
    for call in range(2):
        u = rng.random(m.state_len)
        d_u, d_du = dev(u), torch.full((m.state_len,), np.nan, dtype=torch.float64, device="cuda:0")
        torch.cuda.synchronize()
        if call == 1:
            free_before = torch.cuda.mem_get_info()[0]
        rc = C.lib().gbc_rhs_visco_noalloc(
            mf.nx, mf.nξ, ne, d_st.data_ptr(), d_gm.data_ptr(), ldm, d_g21.data_ptr(), M, d_a.data_ptr(),
            d_b.data_ptr(), d_L.data_ptr(), d_s.data_ptr(), pf.η, pf.vpl, pf.f0, pf.v0, d_gam.data_ptr(),
            d_n.data_ptr(), C.ptr(deps0), d_u.data_ptr(), d_du.data_ptr(), ctypes.c_void_p(stream))
        C.check(rc)
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before  # nothing was allocated
        got = d_du.cpu().numpy()
        ref = m.rhs_flat(u)
        assert np.all(np.isfinite(got))
        np.testing.assert_allclose(got, ref, rtol=RTOL, atol=1e-12 * np.abs(ref).max())


@pytest.mark.gpu
def test_noalloc_replays_from_a_cuda_graph(oracle):
    """The call recorded into a CUDA graph (torch.cuda.graph, global capture mode: an allocation or a
    device-wide synchronisation anywhere in the process would fail the capture) and replayed with
    new states copied into the same buffer: each replay equals the regular entry point."""
    torch = pytest.importorskip("torch")
    from oetqf_gb300 import _capi as C
    from oetqf_gb300.equation import GB300Model
    mf, ma, st, g12, g21, g22, pf, pa = _model(oracle)
    N, ne = mf.nx * mf.nξ, ma.ne
    M = 6 * ne
    m = GB300Model(mf.nx, mf.nξ, ne)
    m.set_gf(C.GBC_GF11_REAL, st)
    m.set_gf(C.GBC_GF12, g12)
    m.set_gf(C.GBC_GF21, g21)
    m.set_gf(C.GBC_GF22, g22)
    m.set_fault_props(pf)
    m.set_mantle_props(pa)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a, dtype=np.float64).reshape(-1), device="cuda:0")
    npad = (N + 31) // 32 * 32
    ldm = npad + M
    gm = np.zeros((M, ldm))
    gm[:, :N], gm[:, npad:npad + M] = g12, g22
    d_st, d_gm, d_g21 = dev(st.reshape(-1, order="F")), dev(gm), dev(g21)
    d_a, d_b, d_L, d_s = (dev(q.reshape(-1, order="F")) for q in (pf.a, pf.b, pf.L, pf.σ))
    d_gam, d_n = dev(pa.γ), dev(pa.n)
    deps0 = np.ascontiguousarray(pa.dϵ0)
    d_u = torch.zeros(m.state_len, dtype=torch.float64, device="cuda:0")
    d_du = torch.zeros(m.state_len, dtype=torch.float64, device="cuda:0")

    def call():
        return C.lib().gbc_rhs_visco_noalloc(
            mf.nx, mf.nξ, ne, d_st.data_ptr(), d_gm.data_ptr(), ldm, d_g21.data_ptr(), M, d_a.data_ptr(),
            d_b.data_ptr(), d_L.data_ptr(), d_s.data_ptr(), pf.η, pf.vpl, pf.f0, pf.v0, d_gam.data_ptr(),
            d_n.data_ptr(), C.ptr(deps0), d_u.data_ptr(), d_du.data_ptr(),
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))

    rng = np.random.default_rng(23)
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):  # one call outside the capture (kernels loaded, scratch address cached)
        d_u.copy_(dev(rng.random(m.state_len)))
        C.check(call())
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        rc = call()
    C.check(rc)
    sentinel = 1.25e300  # every entry of du is written by the replay
    for _ in range(2):
        u = rng.random(m.state_len)
        d_u.copy_(dev(u))
        d_du.fill_(sentinel)
        g.replay()
        torch.cuda.synchronize()
        got = d_du.cpu().numpy()
        ref = m.rhs_flat(u)
        assert not np.any(got == sentinel)
        # the random friction properties can overflow ψ1 on a patch: the same non-finite entries
        np.testing.assert_array_equal(np.isfinite(got), np.isfinite(ref))
        fin = np.isfinite(ref)
        np.testing.assert_allclose(got[fin], ref[fin], rtol=RTOL, atol=1e-12 * np.abs(ref[fin]).max())
