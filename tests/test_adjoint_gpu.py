"""The adjoint sweep (moc_attenuate_adj) against the FP64 CPU adjoint, FP64 central
differences, and torch.autograd.gradcheck through a test-only autograd Function.

Workload: 5,000 tracks with lognormal lengths (about 2,000,000 segments), G = 64,
distributions of the 1M x 64 sweep, seed 4; L = sum w . fine_flux + sum v . psi_out with
w, v ~ N(0, 1)."""
import numpy as np
import pytest

import mocatt
import oracle

pytestmark = pytest.mark.gpu

SEED = 4


def loss_weights(hp, seed=SEED):
    w = np.zeros((hp.R * hp.I, hp.Gs), np.float32)
    v = np.zeros((hp.T, hp.Gs), np.float32)
    w[:, :hp.G] = mocatt.synth_normal(seed, 6, hp.R * hp.I * hp.G).reshape(-1, hp.G)
    v[:, :hp.G] = mocatt.synth_normal(seed, 7, hp.T * hp.G).reshape(-1, hp.G)
    return w, v


def gpu_adjoint(handle, hp, w, v, opts=None):
    import torch

    dp = mocatt.DeviceProblem(hp)
    wt = torch.from_numpy(w).cuda()
    vt = torch.from_numpy(v).cuda()
    ds, dsrc, dpsi = handle.adj(dp, wt, vt, opts)
    assert handle.synchronize() == 0
    # the incoming psi is only read
    np.testing.assert_array_equal(dp.to_host("psi"), hp.psi)
    return ds.cpu().numpy(), dsrc.cpu().numpy(), dpsi.cpu().numpy()


def rel(a, b, floor_frac=1e-3):
    d = np.abs(a.astype(np.float64) - b)
    den = np.maximum(np.abs(b), floor_frac * np.sqrt(np.mean(b * b)))
    r = d / den
    return float(r.max()), float(np.sqrt(np.mean(r * r)))


@pytest.fixture(scope="module")
def adj_problem():
    hp = mocatt.generate(mocatt.WORKLOADS["adjoint_2M_g64"])
    w, v = loss_weights(hp)
    return hp, w, v


@pytest.fixture(scope="module")
def adj_ref(adj_problem):
    hp, w, v = adj_problem
    return oracle.adj_fp64(hp, w.astype(np.float64), v.astype(np.float64))


# -1: one pass per track; 0: tracks of more than 1024 segments cut into 256-segment
# chunks; 32: tracks of more than 128 segments cut into 32-segment chunks
@pytest.mark.parametrize("chunk", [-1, 0, 32])
def test_adjoint_vs_fp64_cpu_adjoint(handle, adj_problem, adj_ref, chunk):
    hp, w, v = adj_problem
    assert 1.8e6 < hp.S < 2.2e6
    ds, dsrc, dpsi = gpu_adjoint(handle, hp, w, v, mocatt.default_opts(track_chunk=chunk))
    ref = adj_ref
    G = hp.G
    out = {k: rel(a[:, :G], ref[r][:, :G]) for k, a, r in (
        ("sigT", ds, "d_sigT"), ("source", dsrc, "d_source"), ("psi_in", dpsi, "d_psi_in"))}
    print(out)
    # measured on GB300: max 1.9e-4 - 2.2e-4 (sigT), 4.2e-4 - 6.1e-4 (source), 4.7e-4
    # (psi_in); RMS 1.7e-6 - 2.3e-6 for every output and chunk length
    for k, (mx, rms) in out.items():
        assert rms <= 1e-5, (k, mx, rms)
        assert mx <= 2e-3, (k, mx, rms)


def test_adjoint_split_keeps_whole_tracks_bitwise(handle, adj_problem):
    """Tracks of at most 4 chunks run the one-pass arithmetic: their dL/dpsi_in equals the
    unsplit run bit for bit."""
    hp, w, v = adj_problem
    _, _, d_one = gpu_adjoint(handle, hp, w, v, mocatt.default_opts(track_chunk=-1))
    _, _, d_cut = gpu_adjoint(handle, hp, w, v, mocatt.default_opts(track_chunk=64))
    whole = np.diff(hp.track_offsets) <= 4 * 64
    assert whole.any() and (~whole).any()
    assert np.array_equal(d_cut[whole], d_one[whole])


def test_packed_pairs_equal_the_one_group_form(handle, adj_problem):
    """Two groups per lane run the packed FP32 form of the recording pass on the pair
    layout of the cell blocks; one group per lane runs the scalar form on blocks in group
    order. Each packed operation rounds as its scalar one, so dL/dpsi_in (carried per
    track, no atomics) is equal bit for bit. The scattered gradients differ only by the
    order of their FP32 atomic sums (measured on GB300: RMS 1.3e-6, max 2.0e-4 apart)."""
    hp, w, v = adj_problem
    one = gpu_adjoint(handle, hp, w, v, mocatt.default_opts(vec=1))
    two = gpu_adjoint(handle, hp, w, v, mocatt.default_opts(vec=2))
    assert np.array_equal(one[2], two[2])
    for a, b in zip(one[:2], two[:2]):
        mx, rms = rel(b[:, :hp.G], a[:, :hp.G].astype(np.float64))
        assert rms <= 1e-5 and mx <= 2e-3, (mx, rms)


def test_adjoint_vs_central_differences(handle, adj_problem):
    """64 random parameters: GPU adjoint and FP64 adjoint vs FP64 central differences
    (h = 1e-6) of the FP64 oracle's loss."""
    hp, w, v = adj_problem
    ds, dsrc, dpsi = gpu_adjoint(handle, hp, w, v)
    w64, v64 = w.astype(np.float64), v.astype(np.float64)
    sig = hp.sigT.astype(np.float64)
    src = hp.source.astype(np.float64)
    psi = hp.psi.astype(np.float64)
    rng = np.random.default_rng(64)
    h = 1e-6
    worst = 0.0
    for n in range(64):
        kind = ("sigT", "source", "psi")[n % 3]
        arr, grad = {"sigT": (sig, ds), "source": (src, dsrc), "psi": (psi, dpsi)}[kind]
        i = int(rng.integers(arr.shape[0]))
        g = int(rng.integers(hp.G))
        args = {"sigT": sig, "source": src, "psi": psi}
        lp_a, lm_a = dict(args), dict(args)
        lp_a[kind] = arr.copy()
        lm_a[kind] = arr.copy()
        lp_a[kind][i, g] += h
        lm_a[kind][i, g] -= h
        lp = oracle.loss_fp64(hp, lp_a["sigT"], lp_a["source"], lp_a["psi"], w64, v64, g)
        lm = oracle.loss_fp64(hp, lm_a["sigT"], lm_a["source"], lm_a["psi"], w64, v64, g)
        fd = (lp - lm) / (2 * h)
        noise = 64 * 2.0 ** -52 * max(abs(lp), abs(lm)) / h
        err = abs(float(grad[i, g]) - fd) / max(abs(fd), 1.0)
        worst = max(worst, err)
        assert abs(float(grad[i, g]) - fd) <= 1e-3 * max(abs(fd), 1.0) + noise, \
            (kind, i, g, float(grad[i, g]), fd)
    print("worst relative deviation from central differences:", worst)


def test_gradcheck_through_autograd_function(handle):
    """A test-only torch.autograd.Function: forward = the FP64 oracle's loss
    L(sigT, source, psi_in) for fixed w, v; backward = the GPU adjoint kernel
    (moc_attenuate_adj). torch.autograd.gradcheck then compares the kernel's gradient
    with FP64 central differences (h = 1e-6) of L, for every input entry of a small
    problem. Tolerance 1e-3 relative: the kernel computes in FP32."""
    import torch

    hp = mocatt.generate(mocatt.WORKLOADS["adjoint_2M_g64"].with_(
        regions=3, groups=4, tracks=6, lognormal=(6.0, 0.5, 1, 20)))
    w, v = loss_weights(hp, seed=9)
    w64, v64 = w.astype(np.float64), v.astype(np.float64)

    class SweepLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, sig, src, psi_in):
            ctx.save_for_backward(sig, src, psi_in)
            L = oracle.loss_fp64(hp, sig.detach().cpu().numpy(), src.detach().cpu().numpy(),
                                 psi_in.detach().cpu().numpy(), w64, v64)
            return torch.tensor(L, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gL):
            sig, src, psi_in = ctx.saved_tensors
            q = hp.copy()
            q.sigT = sig.detach().cpu().numpy().astype(np.float32)
            q.source = src.detach().cpu().numpy().astype(np.float32)
            q.psi = psi_in.detach().cpu().numpy().astype(np.float32)
            ds, dsrc, dpsi = gpu_adjoint(handle, q, w, v)
            g = float(gL)
            return (torch.from_numpy(ds).double() * g, torch.from_numpy(dsrc).double() * g,
                    torch.from_numpy(dpsi).double() * g)

    # padding columns carry no gradient: check the real groups only
    G = hp.G
    sig = torch.from_numpy(hp.sigT.astype(np.float64)).requires_grad_()
    src = torch.from_numpy(hp.source.astype(np.float64)).requires_grad_()
    psi = torch.from_numpy(hp.psi.astype(np.float64)).requires_grad_()
    assert hp.Gs == G  # G = 4: no padding
    # the kernel's FP32 atomic accumulation order varies between runs: nondet_tol
    assert torch.autograd.gradcheck(SweepLoss.apply, (sig, src, psi), eps=1e-6, atol=1e-5,
                                    rtol=1e-3, nondet_tol=1e-3)


def test_gradcheck_split_tracks(handle):
    """gradcheck as above on three tracks of 150-400 segments cut into 32-segment chunks:
    the chunk maps, the psi / lambda scans over chunks and the chunked passes."""
    import torch

    hp = mocatt.generate(mocatt.WORKLOADS["adjoint_2M_g64"].with_(
        regions=3, groups=4, tracks=3, lognormal=(250.0, 0.4, 150, 400)))
    assert hp.S > 4 * 32 and np.diff(hp.track_offsets).min() > 4 * 32
    w, v = loss_weights(hp, seed=11)
    w64, v64 = w.astype(np.float64), v.astype(np.float64)
    opts = mocatt.default_opts(track_chunk=32)

    class SweepLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, sig, src, psi_in):
            ctx.save_for_backward(sig, src, psi_in)
            L = oracle.loss_fp64(hp, sig.detach().cpu().numpy(), src.detach().cpu().numpy(),
                                 psi_in.detach().cpu().numpy(), w64, v64)
            return torch.tensor(L, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gL):
            sig, src, psi_in = ctx.saved_tensors
            q = hp.copy()
            q.sigT = sig.detach().cpu().numpy().astype(np.float32)
            q.source = src.detach().cpu().numpy().astype(np.float32)
            q.psi = psi_in.detach().cpu().numpy().astype(np.float32)
            ds, dsrc, dpsi = gpu_adjoint(handle, q, w, v, opts)
            g = float(gL)
            return (torch.from_numpy(ds).double() * g, torch.from_numpy(dsrc).double() * g,
                    torch.from_numpy(dpsi).double() * g)

    sig = torch.from_numpy(hp.sigT.astype(np.float64)).requires_grad_()
    src = torch.from_numpy(hp.source.astype(np.float64)).requires_grad_()
    psi = torch.from_numpy(hp.psi.astype(np.float64)).requires_grad_()
    # repeated backward calls differ by the FP32 atomic order of the gradient sums: a few
    # hundred terms per entry, so 1e-5 of the largest gradient
    scale = max(float(np.abs(g).max()) for g in gpu_adjoint(handle, hp, w, v, opts))
    assert torch.autograd.gradcheck(SweepLoss.apply, (sig, src, psi), eps=1e-6, atol=1e-5,
                                    rtol=1e-3, nondet_tol=max(1e-3, 1e-5 * scale))


def test_adjoint_rejects_table_mode(handle):
    import torch

    hp = mocatt.generate(mocatt.WORKLOADS["adjoint_2M_g64"].with_(
        regions=3, groups=4, tracks=6, lognormal=(6.0, 0.5, 1, 20)))
    dp = mocatt.DeviceProblem(hp)
    w = torch.zeros_like(dp.fine_flux)
    v = torch.zeros_like(dp.psi)
    with pytest.raises(mocatt.MocError):
        handle.adj(dp, w, v, mocatt.default_opts(exp_mode=mocatt.MOC_EXP_TABLE))
