"""The cost model's tensor-core GEMM (tcgen05.mma kind::f16, BF16 operands, FP32
accumulation in tensor memory) against the same product on the host: BF16-rounded inputs,
FP32 reference; relative tolerance 1e-3 of the largest output for FP32 outputs (the
accumulation order differs), one BF16 ulp more for BF16 outputs."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from tensorsat_gb300 import _device, _native

pytestmark = pytest.mark.gpu


def _gemm(a, b, bias=None, relu=False, out_f32=True):
    lib = _native.lib()
    m, k = a.shape
    n = b.shape[0]
    out = torch.empty((m, n), dtype=torch.float32 if out_f32 else torch.bfloat16, device=a.device)
    _native.check(lib.tsg_cm_gemm_bf16(m, n, k, a.data_ptr(), b.data_ptr(),
                                       None if bias is None else bias.data_ptr(), int(relu),
                                       out.data_ptr(), n, int(out_f32), _device.stream_handle()))
    _native.check(lib.tsg_cm_take_error(_device.stream_handle()))
    return out


@pytest.fixture(params=[0, 1], ids=["tma", "staged"])
def gemm_mode(request):
    lib = _native.lib()
    _native.check(lib.tsg_cm_set_gemm_mode(request.param))
    yield request.param
    _native.check(lib.tsg_cm_set_gemm_mode(DEFAULT_GEMM_MODE))


DEFAULT_GEMM_MODE = 0


@pytest.mark.parametrize("m,n,k", [(128, 64, 64), (128, 128, 64), (256, 128, 256), (1024, 128, 128),
                                   (384, 64, 192)])
def test_gemm_matches_host_product(cuda, gemm_mode, m, n, k):
    g = torch.Generator().manual_seed(m + n + k)
    a = torch.randn(m, k, generator=g).to(torch.bfloat16)
    b = torch.randn(n, k, generator=g).to(torch.bfloat16)
    bias = torch.randn(n, generator=g)
    want = a.float() @ b.float().T + bias
    got = _gemm(a.to(cuda), b.to(cuda), bias.to(cuda)).cpu()
    scale = float(want.abs().max())
    assert float((got - want).abs().max()) <= 1e-3 * scale
    got_relu = _gemm(a.to(cuda), b.to(cuda), bias.to(cuda), relu=True, out_f32=False).cpu().float()
    want_relu = want.clamp(min=0)
    assert float((got_relu - want_relu).abs().max()) <= 1e-3 * scale + 8e-3 * float(want_relu.abs().max())


def test_gemm_rejects_bad_shapes(cuda):
    lib = _native.lib()
    a = torch.zeros(128, 64, dtype=torch.bfloat16, device=cuda)
    out = torch.zeros(128, 256, dtype=torch.float32, device=cuda)
    for m, n, k in [(100, 64, 64), (128, 96, 64), (128, 64, 48), (128, 256, 64)]:
        assert lib.tsg_cm_gemm_bf16(m, n, k, a.data_ptr(), a.data_ptr(), None, 0, out.data_ptr(),
                                    256, 1, None) == _native.TSG_ERR_INVALID_ARGUMENT


def _reference_forward(model, graphs):
    """The same network in plain FP32 torch (operands rounded to BF16 like the kernels)."""
    from tensorsat_gb300 import costmodel as cm

    r = lambda t: t.to(torch.bfloat16).float()
    out = []
    for g in graphs:
        x = r(torch.from_numpy(g["x"]).cuda())
        h = r(torch.relu(x @ r(model.params["w_in"]).T + model.params["b_in"]))
        for l in range(cm.LAYERS):
            c = torch.zeros_like(h)
            for v, ch in enumerate(g["children"]):
                for u in ch:
                    c[v] += h[u]
            hc = torch.cat([h, r(c)], 1)
            h = r(torch.relu(hc @ r(model.params[f"w{l}"]).T + model.params[f"b{l}"]))
        out.append(float(h.sum(0) @ model.params["w_out"] + model.params["b_out"]))
    return np.asarray(out)


def test_cost_model_forward_and_training(cuda):
    """The message-passing network on the tensor cores equals the same network in FP32
    torch within BF16 rounding, and its training kernels (children sums and their
    transpose, weight gradients, Adam) fit a synthetic target: the loss falls well below
    its start."""
    from tensorsat_gb300 import costmodel as cm
    from tensorsat_gb300.contractions.gpu import PRIMES_31, GpuContraction
    from tensorsat_gb300.lang.cuda_rel import CudaRel
    from tensorsat_gb300.lib.sat import CNFInstance

    graphs = []
    for seed in range(24):
        cnf = CNFInstance.random(3, 16 + seed % 8, 4 * (16 + seed % 8), rng=seed)
        c = GpuContraction(CudaRel, cnf.clause_diagram().wiring, target_bits=10, trials=1)
        graphs.append(cm.tree_graph(c, min(4, c.num_slices), PRIMES_31[:3]))
    model = cm.CostModel(seed=1)
    batch = cm.make_batch(graphs[:6], model.device)
    got = model.predict(batch) - model.y_mean
    want = _reference_forward(model, graphs[:6])
    assert np.allclose(got, want, rtol=0.03, atol=0.03 * float(np.abs(want).max()))
    # synthetic target: log of the trees' total index space (a function of the features)
    y = [float(np.log(sum(2.0 ** (32 * g["x"][v, 4]) for v in range(len(g["x"]))
                          if g["x"][v, 1] > 0))) for g in graphs]
    hist = model.fit(graphs, y, epochs=60, batch_trees=8, lr=3e-3)
    assert hist[-1] < 0.25 * hist[0], hist[::10]
