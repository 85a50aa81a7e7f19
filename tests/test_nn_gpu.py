"""The surrogate network's sm_103a kernels (libse2nn.so) against numpy and the
FP64 oracle (oracle/nn_oracle.py): GEMM in every transpose/stride variant,
forward values, loss, gradients of every parameter block, Adam, input assembly.

Tolerances: the GEMM computes in FP32 from BF16 operands, so against an FP64
product of the same BF16-rounded operands it agrees to FP32 accumulation error
(relative 1e-5).  The network stores activations in BF16 (8-bit mantissa), so
outputs agree with the FP64 oracle to a relative L2 of 2e-2 and gradients to
6e-2 per parameter block (cosine similarity >= 0.998 overall).
"""
import numpy as np
import pytest

from oracle import nn_oracle as NO

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from se2dr_fork_gb300 import nn as N  # noqa: E402

SMALL = N.Config(ny=32, nx=32, cin=16, width=16, modes=4, layers=2, nrec=4, nout=64, hidden=32, max_batch=4)
REC_SMALL = [3, 10, 17, 30]


@pytest.fixture(scope="module", autouse=True)
def _built(nn_lib):
    return nn_lib


def bf16_round(a):
    return torch.tensor(np.asarray(a, dtype=np.float32)).to(torch.bfloat16).float().numpy().astype(np.float64)


def dev_bf16(a):
    return torch.tensor(np.asarray(a, dtype=np.float32)).to(torch.bfloat16).cuda()


def rel(x, ref):
    return float(np.linalg.norm(np.asarray(x, dtype=np.float64) - ref) / max(np.linalg.norm(ref), 1e-300))


def oracle_cfg(c: N.Config) -> NO.Config:
    return NO.Config(**{f: getattr(c, f) for f in NO.Config.__dataclass_fields__})


@pytest.mark.parametrize("tA,tB", [(0, 0), (0, 1), (1, 0), (1, 1)])
@pytest.mark.parametrize("M,N_,K,batch,pad", [(1, 1, 1, 1, 0), (37, 70, 45, 3, 3), (130, 64, 128, 2, 8),
                                               (64, 2048, 256, 1, 0), (5, 9, 300, 4, 1), (200, 40, 16, 5, 0)])
def test_gemm_matches_numpy(tA, tB, M, N_, K, batch, pad):
    rng = np.random.default_rng(M * 7 + N_ + K + batch)
    ra, ca = (K, M) if tA else (M, K)
    rb, cb = (N_, K) if tB else (K, N_)
    lda, ldb = ca + pad, cb + pad
    A = bf16_round(rng.standard_normal((batch, ra, lda)))
    B = bf16_round(rng.standard_normal((batch, rb, ldb)))
    C0 = rng.standard_normal((batch, M, N_))
    Ad, Bd = dev_bf16(A), dev_bf16(B)
    Cd = torch.tensor(C0, dtype=torch.float32).cuda()
    N.gemm(Ad, Bd, Cd, M, N_, K, batch, lda, ldb, N_, ra * lda, rb * ldb, M * N_, tA, tB, alpha=1.5, beta=0.5)
    torch.cuda.synchronize()
    opA = A[:, :, :ca].transpose(0, 2, 1) if tA else A[:, :, :ca]
    opB = B[:, :, :cb].transpose(0, 2, 1) if tB else B[:, :, :cb]
    ref = 1.5 * np.einsum("bmk,bkn->bmn", opA, opB) + 0.5 * C0.astype(np.float32)
    assert rel(Cd.cpu().numpy(), ref) < 1e-5


def test_gemm_shared_operand_batches():
    rng = np.random.default_rng(9)
    A = bf16_round(rng.standard_normal((32, 128)))        # shared by every batch (stride 0)
    B = bf16_round(rng.standard_normal((6, 128, 64)))
    Cd = torch.zeros(6, 32, 64, device="cuda")
    N.gemm(dev_bf16(A), dev_bf16(B), Cd, 32, 64, 128, 6, 128, 64, 64, 0, 128 * 64, 32 * 64)
    torch.cuda.synchronize()
    assert rel(Cd.cpu().numpy(), np.einsum("mk,bkn->bmn", A, B)) < 1e-5


@pytest.mark.parametrize("M,N_,K,tB,pad", [(128, 16, 16, 0, 0), (1000, 64, 64, 0, 8), (1000, 64, 64, 1, 0),
                                            (16384, 64, 64, 0, 0), (4096, 128, 128, 1, 8), (777, 16, 128, 0, 0),
                                            (2048, 128, 64, 0, 0), (4096, 128, 16, 0, 8)])
def test_gemm_tensor_core_path_matches_numpy_and_mma(M, N_, K, tB, pad):
    """Row GEMMs that qualify for the tcgen05 kernel (one batch, k-contiguous A, M >= 128,
    K and N multiples of 16 up to 128, ragged row tiles included; mode 2 sends every one
    there) agree with numpy and
    with the mma.sync kernel to FP32 accumulation error; the launch counters show which
    kernel ran, and no bounded wait expired."""
    rng = np.random.default_rng(M + 3 * N_ + 7 * K + tB)
    lda = K + pad
    rb, cb = (N_, K) if tB else (K, N_)
    ldb = cb + pad
    A = bf16_round(rng.standard_normal((M, lda)))
    B = bf16_round(rng.standard_normal((rb, ldb)))
    C0 = rng.standard_normal((M, N_))
    Ad, Bd = dev_bf16(A), dev_bf16(B)
    opB = B[:, :cb].T if tB else B[:, :cb]
    ref = 1.5 * (A[:, :K] @ opB) + 0.5 * C0.astype(np.float32)
    out = {}
    for tc in (True, False):
        N.set_tensor_path(2 if tc else 0)
        before = N.tensor_path_info()
        Cd = torch.tensor(C0, dtype=torch.float32).cuda()
        N.gemm(Ad, Bd, Cd, M, N_, K, 1, lda, ldb, N_, 0, 0, 0, 0, tB, alpha=1.5, beta=0.5)
        torch.cuda.synchronize()
        after = N.tensor_path_info()
        key = "tcgen05_launches" if tc else "mma_sync_launches"
        assert after[key] == before[key] + 1, (before, after)
        out[tc] = Cd.cpu().numpy()
    N.set_tensor_path(1)
    assert not N.tensor_path_info()["wait_expired"]
    assert rel(out[True], ref) < 1e-5, rel(out[True], ref)
    assert rel(out[True], out[False]) < 1e-5


def run_case(cfg, rec_x, B, seed):
    net = N.Network(cfg, seed=seed)
    net.set_receivers(rec_x)
    rng = np.random.default_rng(seed + 100)
    x = np.zeros((B, cfg.ny, cfg.nx, cfg.cin))
    x[..., :6] = rng.standard_normal((B, cfg.ny, cfg.nx, 6))
    x = bf16_round(x)
    t = rng.standard_normal((B, cfg.nrec, cfg.nout))
    out = torch.zeros(B, cfg.nrec, cfg.nout, device="cuda")
    loss = net.loss_grad(dev_bf16(x), torch.tensor(t, dtype=torch.float32).cuda(), out)
    p = net.params().astype(np.float64)
    g = net.grads().astype(np.float64)
    oloss, og, oout = NO.loss_grad(p, x, t, oracle_cfg(cfg), rec_x)
    return net, x, t, loss, g, out.cpu().numpy(), oloss, og, oout


def check_against_oracle(cfg, loss, g, out, oloss, og, oout):
    assert rel(out, oout) < 2e-2, rel(out, oout)
    assert abs(loss - oloss) < 2e-2 * oloss
    lay, _ = NO.layout(oracle_cfg(cfg))
    errs = {}
    for name, (o, s) in lay.items():
        n = int(np.prod(s))
        errs[name] = rel(g[o:o + n], og[o:o + n])
    print({k: "%.1e" % v for k, v in errs.items()})
    assert max(errs.values()) < 6e-2, errs
    cos = float(g @ og / (np.linalg.norm(g) * np.linalg.norm(og)))
    assert cos > 0.998, cos


def test_forward_loss_and_gradients_vs_oracle_small():
    net, x, t, loss, g, out, oloss, og, oout = run_case(SMALL, REC_SMALL, 3, seed=1)
    check_against_oracle(SMALL, loss, g, out, oloss, og, oout)
    # the forward entry point gives the same output as the loss pass
    o2 = torch.zeros(3, SMALL.nrec, SMALL.nout, device="cuda")
    net.forward(dev_bf16(x), o2)
    torch.cuda.synchronize()
    assert np.array_equal(o2.cpu().numpy(), out)


def test_forward_loss_and_gradients_vs_oracle_full_size():
    cfg = N.Config(max_batch=2)
    rec = [int((2 * r + 1) * 128 / 32) for r in range(16)]
    _, _, _, loss, g, out, oloss, og, oout = run_case(cfg, rec, 2, seed=2)
    check_against_oracle(cfg, loss, g, out, oloss, og, oout)


def test_adam_step_vs_oracle():
    net, x, t, loss, g, out, *_ = run_case(SMALL, REC_SMALL, 2, seed=4)
    p = net.params().astype(np.float64)
    net.adam_step(1e-3, 0.9, 0.999, 1e-8, 1e-4)
    q = net.params().astype(np.float64)
    ref, _, _ = NO.adam(p, g, np.zeros_like(p), np.zeros_like(p), 1, 1e-3, 0.9, 0.999, 1e-8, 1e-4)
    np.testing.assert_allclose(q, ref, rtol=1e-5, atol=1e-7)


def test_build_inputs_vs_oracle():
    cfg = SMALL
    net = N.Network(cfg, seed=0)
    rng = np.random.default_rng(5)
    mats = np.stack([rng.uniform(3000, 6000, (5, cfg.ny, cfg.nx)), rng.uniform(1600, 3700, (5, cfg.ny, cfg.nx)),
                     rng.uniform(2000, 3000, (5, cfg.ny, cfg.nx))], axis=-1)
    src = rng.uniform(0, cfg.nx, (5, 2))
    idx = np.array([4, 0, 2], dtype=np.int32)
    x = torch.zeros(3, cfg.ny, cfg.nx, cfg.cin, dtype=torch.bfloat16, device="cuda")
    net.build_inputs(torch.tensor(mats, dtype=torch.float32).cuda(), torch.tensor(src, dtype=torch.float32).cuda(),
                     torch.tensor(idx).cuda(), 2.0, x)
    torch.cuda.synchronize()
    ref = NO.build_inputs(mats, src, idx, oracle_cfg(cfg), 2.0)
    got = x.float().cpu().numpy()
    assert np.max(np.abs(got - ref)) < 1.6e-2
    assert np.all(got[..., 6:] == 0)
    tg = torch.tensor(rng.standard_normal((5, cfg.nrec, cfg.nout)), dtype=torch.float32).cuda()
    rows = torch.zeros(3, cfg.nrec, cfg.nout, device="cuda")
    net.gather_targets(tg, torch.tensor(idx).cuda(), rows)
    torch.cuda.synchronize()
    assert np.array_equal(rows.cpu().numpy(), tg.cpu().numpy()[idx])


def test_training_reduces_loss_on_a_teacher():
    """A student trained with the GPU kernels fits the outputs of a teacher network."""
    cfg = SMALL
    teacher, student = N.Network(cfg, seed=11), N.Network(cfg, seed=12)
    for n in (teacher, student):
        n.set_receivers(REC_SMALL)
    rng = np.random.default_rng(13)
    xs = np.zeros((16, cfg.ny, cfg.nx, cfg.cin))
    xs[..., :6] = rng.standard_normal((16, cfg.ny, cfg.nx, 6))
    xd = dev_bf16(xs)
    t = torch.zeros(16, cfg.nrec, cfg.nout, device="cuda")
    for b in range(0, 16, 4):
        teacher.forward(xd[b:b + 4], t[b:b + 4])
    losses = []
    for step in range(300):
        b = (step % 4) * 4
        losses.append(student.loss_grad(xd[b:b + 4], t[b:b + 4]))
        student.adam_step(2e-3)
    first, last = np.mean(losses[:4]), np.mean(losses[-4:])
    print("loss", first, "->", last)
    assert last < 0.2 * first
