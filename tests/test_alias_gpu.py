"""Device alias-table build and sampling through the C ABI.

Reference mode must reproduce the reference's generateAliasTable bit for bit
(golden tables written from the reference's own code, plus the 200,000-weight
stress table and a 65,536-emitter table); sweep mode must reproduce the oracle's
CPU restatement of the sweep build bit for bit; sampling must reproduce sample().
"""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def device_build(ctx, native, w, mode):
    w = np.ascontiguousarray(w, np.float32)
    n = w.size
    dw = torch.from_numpy(w).cuda() if n else torch.empty(1, device="cuda")
    out = torch.zeros(max(n, 1) * 5, dtype=torch.int32, device="cuda")
    ctx.alias_build(dw, n, out, mode)
    torch.cuda.synchronize()
    return out.cpu().numpy()[: n * 5].view(native.ALIAS_DTYPE)


def test_reference_mode_matches_reference_tables(native, ctx, golden):
    g = golden("alias.npz")
    off = g["offsets"]
    for c in range(len(off) - 1):
        w = g["weights"][off[c]:off[c + 1]]
        tab = device_build(ctx, native, w, native.DR_ALIAS_REFERENCE)
        sl = slice(off[c], off[c + 1])
        for k in ("p_A", "pdf_A", "pdf_B"):
            assert np.array_equal(tab[k].view(np.uint32), g[k][sl].view(np.uint32)), f"case {c} {k}"
        assert np.array_equal(tab["A"], g["A"][sl]) and np.array_equal(tab["B"], g["B"][sl]), f"case {c}"


def test_reference_mode_stress_and_emitter_tables(native, ctx, oracle, golden):
    g = golden("alias.npz")
    w = oracle.lognormal_input(200000, 42)
    tab = device_build(ctx, native, w, native.DR_ALIAS_REFERENCE)
    assert hashlib.sha256(tab.tobytes()).digest() == g["stress_table_sha"].tobytes()
    tab = device_build(ctx, native, g["emitter_weights"], native.DR_ALIAS_REFERENCE)
    assert hashlib.sha256(tab.tobytes()).digest() == g["emitter_table_sha"].tobytes()


@pytest.mark.parametrize("n", [1, 2, 3, 7, 100, 511, 512, 513, 1000, 4096, 65536, 200000, 1 << 20])
def test_sweep_mode_matches_oracle(native, ctx, oracle, n):
    rng = np.random.default_rng(n)
    w = rng.lognormal(0, 1.5, n).astype(np.float32)
    if n > 10:
        w[rng.random(n) < 0.2] = 0.0
    tab = device_build(ctx, native, w, native.DR_ALIAS_SWEEP)
    ref = oracle.alias_build_sweep(w)
    assert tab.tobytes() == ref.tobytes()


def test_sweep_mode_golden_cases_and_edge_inputs(native, ctx, oracle, golden):
    g = golden("alias.npz")
    off = g["offsets"]
    cases = [g["weights"][off[c]:off[c + 1]] for c in range(len(off) - 1)]
    cases += [np.array([np.nan, 1.0, np.inf, -np.inf, 2.0], np.float32), np.full(10, 1e-30, np.float32),
              np.array([3e38, 3e38, 1e-38], np.float32)]
    for c, w in enumerate(cases):
        tab = device_build(ctx, native, w, native.DR_ALIAS_SWEEP)
        assert tab.tobytes() == oracle.alias_build_sweep(w).tobytes(), f"case {c}"


@pytest.mark.parametrize("mode", [0, 1])
def test_device_sampling_matches_oracle(native, ctx, oracle, mode):
    rng = np.random.default_rng(3)
    n = 5000
    w = rng.lognormal(0, 1, n).astype(np.float32)
    tab = device_build(ctx, native, w, mode)
    u = rng.random((100000, 2)).astype(np.float32)
    u[:3] = [[0, 0], [np.nextafter(np.float32(1), np.float32(0)), 1.0], [0.5, 0.5]]
    dt = torch.from_numpy(tab.view(np.int32).reshape(-1).copy()).cuda()
    du = torch.from_numpy(u.reshape(-1).copy()).cuda()
    idx = torch.empty(len(u), dtype=torch.int32, device="cuda")
    pdf = torch.empty(len(u), dtype=torch.float32, device="cuda")
    native.alias_sample(dt, n, du, len(u), idx, pdf)
    torch.cuda.synchronize()
    idx, pdf = idx.cpu().numpy(), pdf.cpu().numpy()
    for k in range(0, len(u), 97):
        i, p = oracle.alias_sample(tab, float(u[k, 0]), float(u[k, 1]))
        assert idx[k] == i and pdf[k] == np.float32(p)
    # empirical frequencies follow the weights
    freq = np.bincount(idx, minlength=n) / len(u)
    assert np.abs(freq - w / w.sum()).max() < 2e-3
