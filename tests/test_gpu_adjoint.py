"""Adjoint gradients on the GPU (batched kernels behind torch.autograd.Function) against
the reference's parameter-shift gradient and the FP64 oracle's central differences."""
import numpy
import pytest
import torch

from conftest import load_npz
from qip_gb300 import adjoint
from test_adjoint_cpu import oracle_energy

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("statetype,atol", [(torch.complex128, 1e-10), (torch.complex64, 2e-5)])
def test_adjoint_matches_reference_parameter_shift(statetype, atol):
    d = load_npz("workloads.npz")[0]
    n, layers = (int(x) for x in d["ansatz_ps_shape"])
    th = torch.tensor(d["ansatz_ps_thetas"], device="cuda")
    e, g = adjoint.energy_and_grad(th, adjoint.Ansatz(n, layers), statetype)
    numpy.testing.assert_allclose(e.cpu().numpy(), d["ansatz_ps_energies"], atol=atol)
    numpy.testing.assert_allclose(g.cpu().numpy(), d["ansatz_ps_grads"], atol=atol * 10)


def test_adjoint_matches_oracle_finite_differences():
    n, layers = 9, 3
    a = adjoint.Ansatz(n, layers)
    rng = numpy.random.default_rng(5)
    th = rng.uniform(0, 2 * numpy.pi, (2, a.nparams))
    e, g = adjoint.energy_and_grad(torch.tensor(th, device="cuda"), a, torch.complex128)
    for b in range(2):
        assert abs(e[b].item() - oracle_energy(th[b], n, layers)) < 1e-10
        for j in rng.choice(a.nparams, 12, replace=False):
            tp, tm = th[b].copy(), th[b].copy()
            tp[j] += 1e-3
            tm[j] -= 1e-3
            fd = (oracle_energy(tp, n, layers) - oracle_energy(tm, n, layers)) / 2e-3
            assert abs(g[b, j].item() - fd) < 1e-5


def test_adjoint_upstream_gradient_and_batch_independence():
    n, layers = 8, 2
    a = adjoint.Ansatz(n, layers)
    th = torch.tensor(numpy.random.default_rng(2).uniform(0, 6, (4, a.nparams)), device="cuda", requires_grad=True)
    e = adjoint.SumZExpectation.apply(th, a, torch.complex128)
    w = torch.tensor([1.0, -2.0, 0.5, 0.0], device="cuda", dtype=torch.float64)
    (e * w).sum().backward()
    e1, g1 = adjoint.energy_and_grad(th.detach()[1:2], a, torch.complex128)
    numpy.testing.assert_allclose(th.grad[1].cpu().numpy(), -2.0 * g1[0].cpu().numpy(), atol=1e-11)
    assert torch.all(th.grad[3] == 0)


@pytest.mark.parametrize("statetype,rtol", [(torch.complex128, 1e-11), (torch.complex64, 2e-5)])
def test_segmented_sweeps_match_per_gate_sweeps(statetype, rtol):
    """Segments (13 / 12 local bits: 8 / 16 chunks per set at n=16) give the per-gate
    energies and gradients; both parametrisations of the autograd Function agree."""
    n, layers, B = 16, 3, 3
    a = adjoint.Ansatz(n, layers)
    assert len(adjoint.plan_segments(a, adjoint.local_bits(statetype))) > 1
    th = torch.tensor(numpy.random.default_rng(11).uniform(0, 2 * numpy.pi, (B, a.nparams)), device="cuda")
    e1, g1 = adjoint.energy_and_grad(th, a, statetype, segmented=True)
    e0, g0 = adjoint.energy_and_grad(th, a, statetype, segmented=False)
    scale = float(torch.max(torch.abs(g0)))
    numpy.testing.assert_allclose(e1.cpu().numpy(), e0.cpu().numpy(), atol=rtol * n)
    numpy.testing.assert_allclose(g1.cpu().numpy(), g0.cpu().numpy(), atol=rtol * scale * 10)


@pytest.mark.parametrize("n,layers,B", [(14, 3, 4), (16, 4, 3)])
def test_tensor_core_adjoint_matches_fp64_path(n, layers, B):
    """Tensor-core adjoint (complex64, split-bf16 block products, tensor-core
    correlations, FP64 walks) against the complex128 segment kernels: energies within
    1e-5, gradients within 5e-5 (measured: 1.3e-6 and 8e-6 at n=14)."""
    a = adjoint.Ansatz(n, layers)
    th = torch.tensor(numpy.random.default_rng(n).uniform(0, 2 * numpy.pi, (B, a.nparams)), device="cuda")
    e1, g1 = adjoint.energy_and_grad(th, a, torch.complex64, "tensor")
    e0, g0 = adjoint.energy_and_grad(th, a, torch.complex128, "segmented")
    assert len(adjoint.tensor_core_plan(a).blocks) > 1
    numpy.testing.assert_allclose(e1.cpu().numpy(), e0.cpu().numpy(), atol=1e-5)
    numpy.testing.assert_allclose(g1.cpu().numpy(), g0.cpu().numpy(), atol=5e-5)


def test_tensor_core_adjoint_three_launch_backward():
    """Blocks whose placement class is pinned to the shuffle mode take the backward path
    of correlation kernel + walk + two block launches (the fused pass covers the direct,
    prefix and pair modes); gradients against the complex128 segment kernels."""
    from qip_gb300 import GpuBackend, _native as nat

    n, layers, B = 15, 3, 3
    a = adjoint.Ansatz(n, layers)
    # Every class of the ansatz is pinned (modes recorded by earlier tuning in this process
    # would otherwise decide): shuffle where it applies, direct elsewhere.
    lows, pins = set(), {}
    for qs, _ in adjoint.block_partition(a):
        low = sum(1 << (n - 1 - q) for q in qs if n - 1 - q < 7)
        lows.add(low)
        pins[low] = 2 if 1 <= bin(low & 0x1F).count("1") <= 5 else 0
    assert 2 in pins.values() and 0 in pins.values()
    lib = nat.load()
    st = GpuBackend.make_state(13, [], [], statetype=numpy.complex64, fusion=True, autotune=False)
    adjoint._TC_PLANS.pop((n, layers), None)
    try:
        for low in lows:
            nat.check(lib.qsv_set_block_mode(st.handle, 6, low, pins[low]), st.handle, "set_block_mode")
        th = torch.tensor(numpy.random.default_rng(7).uniform(0, 2 * numpy.pi, (B, a.nparams)), device="cuda")
        e1, g1 = adjoint.energy_and_grad(th, a, torch.complex64, "tensor")
        e0, g0 = adjoint.energy_and_grad(th, a, torch.complex128, "segmented")
        plan = adjoint.tensor_core_plan(a)
        assert 0 < plan.fused_blocks < len(plan.blocks)  # both backward paths in one sweep
    finally:
        for low in lows:
            lib.qsv_set_block_mode(st.handle, 6, low, -1)
        adjoint._TC_PLANS.pop((n, layers), None)
        st.close()
    numpy.testing.assert_allclose(e1.cpu().numpy(), e0.cpu().numpy(), atol=1e-5)
    numpy.testing.assert_allclose(g1.cpu().numpy(), g0.cpu().numpy(), atol=5e-5)


def test_tensor_core_adjoint_upstream_gradient_and_defaults():
    """complex64 at n >= 13 takes the tensor cores by default; the upstream gradient
    scales each set's row; a set with weight 0 gets zeros."""
    n, layers = 13, 2
    a = adjoint.Ansatz(n, layers)
    th = torch.tensor(numpy.random.default_rng(4).uniform(0, 6, (3, a.nparams)), device="cuda", requires_grad=True)
    e = adjoint.SumZExpectation.apply(th, a, torch.complex64)
    w = torch.tensor([2.0, 0.0, -1.0], device="cuda", dtype=torch.float64)
    (e * w).sum().backward()
    _, g = adjoint.energy_and_grad(th.detach(), a, torch.complex64, "tensor")
    numpy.testing.assert_allclose(th.grad[0].cpu().numpy(), 2 * g[0].cpu().numpy(), atol=1e-12)
    numpy.testing.assert_allclose(th.grad[2].cpu().numpy(), -g[2].cpu().numpy(), atol=1e-12)
    assert torch.all(th.grad[1] == 0)
    with pytest.raises(ValueError):
        adjoint.energy_and_grad(th.detach(), adjoint.Ansatz(8, 2), torch.complex64, "tensor")


def test_config5_full_size_against_central_differences():
    """Config 5 at its own size: n=24, 20 layers (960 angles), 64 parameter sets,
    complex64 adjoint gradients (the default: tensor cores) and the CUDA-core segment
    kernels; seeded (set, angle) pairs against central differences
    (h=1e-3) of the complex128 energy (per-gate FP64 kernels, pinned to the oracle and
    the reference's parameter-shift gradients at small n by the tests above)."""
    n, layers, B = 24, 20, 64
    a = adjoint.Ansatz(n, layers)
    th = torch.tensor(numpy.random.default_rng(2025).uniform(0, 2 * numpy.pi, (B, a.nparams)), device="cuda")
    e, g = adjoint.energy_and_grad(th, a, torch.complex64)
    es, gs = adjoint.energy_and_grad(th, a, torch.complex64, "segmented")
    assert e.shape == (B,) and g.shape == (B, a.nparams)
    assert torch.all(torch.isfinite(g))
    numpy.testing.assert_allclose(g.cpu().numpy(), gs.cpu().numpy(), atol=5e-6)
    rng = numpy.random.default_rng(31)
    pairs = [(int(rng.integers(B)), int(j)) for j in rng.choice(a.nparams, 6, replace=False)]
    pairs += [(0, 0), (B - 1, a.nparams - 1)]
    for b, j in pairs:
        tp, tm = th[b:b + 1].clone(), th[b:b + 1].clone()
        tp[0, j] += 1e-3
        tm[0, j] -= 1e-3
        with torch.no_grad():
            ep = adjoint.SumZExpectation.apply(tp, a, torch.complex128)
            em = adjoint.SumZExpectation.apply(tm, a, torch.complex128)
        fd = float((ep - em).item() / 2e-3)
        assert abs(g[b, j].item() - fd) < 1e-5 + 1e-3 * abs(fd), (b, j, g[b, j].item(), fd)
        assert abs(gs[b, j].item() - fd) < 1e-6 + 1e-4 * abs(fd), (b, j, gs[b, j].item(), fd)
    with torch.no_grad():
        e128 = adjoint.SumZExpectation.apply(th[:2].clone(), a, torch.complex128)
    numpy.testing.assert_allclose(e[:2].cpu().numpy(), e128.cpu().numpy(), atol=2e-5)


@pytest.mark.parametrize("cdtype,atol", [(torch.complex128, 1e-15), (torch.complex64, 1e-7)])
def test_device_rotation_matrices_match_the_circuit_generator(cdtype, atol):
    """qsv_batch_rotation_matrices: U and U^+ of every gate and set against the matrices
    of circuits.ansatz_layers (RY, RZ, and X for the CNOTs)."""
    from qip_gb300 import circuits

    n, layers, B = 5, 2, 3
    a = adjoint.Ansatz(n, layers)
    th = numpy.random.default_rng(0).uniform(0, 6, (B, a.nparams))
    U, Ud = adjoint.gate_matrices(a, torch.tensor(th, device="cuda"), cdtype)
    U, Ud = U.cpu().numpy(), Ud.cpu().numpy()
    for b in range(B):
        dicts = circuits.ansatz_layers(n, layers, th[b])
        for g, d in enumerate(dicts):
            (key, m), = d.items()
            want = m.m if getattr(m, "_kron_struct", None) == 2 else m
            numpy.testing.assert_allclose(U[g, b].reshape(2, 2), want, atol=atol)
            numpy.testing.assert_allclose(Ud[g, b].reshape(2, 2), numpy.conj(want).T, atol=atol)
