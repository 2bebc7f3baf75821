"""GPU: the adjoints of the CGH sums (olg_cgh_fresnel_adjoint_c64,
olg_cgh_exact_adjoint_c64), the transposed sums g = A^H G.

Checked three ways: against the FP64 oracle's transposed sums
(olc_cgh_fresnel_adjoint / olc_cgh_exact_adjoint) at the FP32 gate, by the
dot-product identity <A x, G> = <x, A^H G> on the full CGH workload
(1920 x 1080, 10,000 points), and wrapped in a torch.autograd.Function (in
this test only) whose gradient matches torch autograd through a dense
FP64 matrix of the same kernel."""
import numpy as np
import pytest
import torch

import oracle as O
import openol_gb300 as og
from conftest import rel_l2
from test_gpu_cgh import config2_points

pytestmark = pytest.mark.gpu
TOL = 1e-5
FWD = {"fresnel": og.cgh_fresnel, "exact": og.cgh_exact, "fresnel_gemm": og.cgh_fresnel_gemm}
ADJ = {"fresnel": og.cgh_fresnel_adjoint, "exact": og.cgh_exact_adjoint, "fresnel_gemm": og.cgh_fresnel_adjoint_gemm}
ORA = {"fresnel": O.cgh_fresnel_adjoint, "exact": O.cgh_exact_adjoint, "fresnel_gemm": O.cgh_fresnel_adjoint}


def small_case(seed, n=700, ny=100, nx=130, p=8e-6):
    """Edges on purpose: n is not a multiple of the 256-point chunk, and
    neither side of the hologram a multiple of the 16 x 16 subtile."""
    rng = np.random.default_rng(seed)
    pts = np.stack([rng.random(n) * nx * p, rng.random(n) * ny * p, 0.02 + 0.01 * rng.random(n)], 1)
    G = (rng.standard_normal((ny, nx)) + 1j * rng.standard_normal((ny, nx))).astype(np.complex64)
    return pts.astype(np.float32), G


@pytest.mark.parametrize("form", ["fresnel", "exact", "fresnel_gemm"])
def test_cgh_adjoint_vs_oracle(form):
    pts, G = small_case({"fresnel": 7, "exact": 8, "fresnel_gemm": 10}[form])
    ny, nx, p, lam = G.shape[0], G.shape[1], 8e-6, 532e-9
    g = ADJ[form](og.gObject(pts), torch.from_numpy(G).cuda(), ny=ny, nx=nx, py=p, px=p, lam=lam)
    torch.cuda.synchronize()
    ref = ORA[form](pts.astype(np.float64), G.astype(np.complex128), p, p, lam)
    assert rel_l2(g.cpu().numpy(), ref) < TOL


@pytest.mark.parametrize("form", ["fresnel", "fresnel_gemm"])
def test_cgh_adjoint_accumulates(form):
    pts, G = small_case(9, n=300, ny=48, nx=64)
    obj, Gd = og.gObject(pts), torch.from_numpy(G).cuda()
    kw = dict(ny=48, nx=64, py=8e-6, px=8e-6, lam=532e-9)
    once = ADJ[form](obj, Gd, **kw)
    g = once.clone()
    ADJ[form](obj, Gd, g, accumulate=True, **kw)
    torch.cuda.synchronize()
    assert rel_l2(g.cpu().numpy(), 2 * once.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("pairs", [False, True], ids=["single", "pairs"])
def test_cgh_adjoint_gemm_scale_and_agreement(pairs):
    """The tensor-core adjoint scales G by a power of two to keep its f16
    operands in range: a field far outside f16's range (1e8) and a tiny one
    (1e-9) give the same g up to that factor, and the two Fresnel adjoints
    agree on an uneven shape (n, nx, ny not multiples of the tiles), in both
    GEMM tile forms."""
    pts, G = small_case(12, n=517, ny=77, nx=133)
    obj = og.gObject(pts)
    kw = dict(ny=77, nx=133, py=8e-6, px=8e-6, lam=532e-9)
    ref = og.cgh_fresnel_adjoint(obj, torch.from_numpy(G).cuda(), **kw).cpu().numpy()
    prev = og.cgh_gemm_pairs(pairs)
    try:
        for scale in (1.0, 1e8, 1e-9):
            Gs = torch.from_numpy((G * scale).astype(np.complex64)).cuda()
            g = og.cgh_fresnel_adjoint_gemm(obj, Gs, **kw)
            torch.cuda.synchronize()
            assert rel_l2(g.cpu().numpy() / scale, ref) < TOL, scale
    finally:
        og.cgh_gemm_pairs(prev)


@pytest.mark.parametrize("form", ["fresnel", "exact", "fresnel_gemm"])
def test_cgh_adjoint_dot_product_workload(form):
    """<A x, G> = <x, A^H G> on the CGH workload: 10,000 points with complex
    amplitudes x_j = a_j e^{i phi_j}, 1920 x 1080 hologram, random G."""
    pts, amp, ph = config2_points(10000)
    ny, nx, p, lam = 1080, 1920, 8e-6, 532e-9
    obj = og.gObject(pts)
    U = torch.zeros((ny, nx), dtype=torch.complex64, device="cuda")
    FWD[form](obj, U, ny=ny, nx=nx, py=p, px=p, lam=lam, amp=torch.from_numpy(amp).cuda(),
              phase0=torch.from_numpy(ph).cuda())
    gen = torch.Generator(device="cuda").manual_seed(11)
    G = torch.complex(torch.randn((ny, nx), device="cuda", generator=gen),
                      torch.randn((ny, nx), device="cuda", generator=gen))
    g = ADJ[form](obj, G, ny=ny, nx=nx, py=p, px=p, lam=lam)
    torch.cuda.synchronize()
    Ax = U.cpu().numpy().astype(np.complex128)
    Gh = G.cpu().numpy().astype(np.complex128)
    x = amp.astype(np.float64) * np.exp(1j * ph.astype(np.float64))
    lhs = np.vdot(Ax, Gh)
    rhs = np.vdot(x, g.cpu().numpy().astype(np.complex128))
    scale = np.linalg.norm(Ax) * np.linalg.norm(Gh)
    assert abs(lhs - rhs) / scale < 1e-6, (lhs, rhs)


class CghFresnel(torch.autograd.Function):
    """Fresnel CGH as a differentiable map from complex point amplitudes to
    the hologram; backward is the hand-written adjoint kernel (test harness
    only: the library itself exports the C-ABI, not autograd)."""

    @staticmethod
    def forward(ctx, c, obj, ny, nx, p, lam):
        ctx.meta = (obj, ny, nx, p, lam)
        U = torch.zeros((ny, nx), dtype=torch.complex64, device=c.device)
        og.cgh_fresnel(obj, U, ny=ny, nx=nx, py=p, px=p, lam=lam, amp=c.abs().contiguous(),
                       phase0=torch.angle(c).contiguous())
        return U

    @staticmethod
    def backward(ctx, grad_U):
        obj, ny, nx, p, lam = ctx.meta
        g = og.cgh_fresnel_adjoint(obj, grad_U.contiguous(), ny=ny, nx=nx, py=p, px=p, lam=lam)
        return g, None, None, None, None, None


def test_cgh_adjoint_autograd_matches_dense_fp64():
    n, ny, nx, p, lam = 40, 24, 32, 8e-6, 532e-9
    rng = np.random.default_rng(5)
    pts = np.stack([rng.random(n) * nx * p, rng.random(n) * ny * p, 0.02 + 0.01 * rng.random(n)], 1)
    pts = pts.astype(np.float32)
    c0 = (0.5 + rng.random(n)) * np.exp(2j * np.pi * rng.random(n))
    T = rng.random((ny, nx)) * np.exp(2j * np.pi * rng.random((ny, nx)))
    # GPU: the custom Function
    c = torch.tensor(c0, dtype=torch.complex64, device="cuda", requires_grad=True)
    U = CghFresnel.apply(c, og.gObject(pts), ny, nx, p, lam)
    loss = (U - torch.from_numpy(T.astype(np.complex64)).cuda()).abs().pow(2).sum()
    loss.backward()
    # reference: dense FP64 matrix of the unit kernels, torch autograd on the CPU
    A = np.stack([O.cgh_fresnel(pts[j:j + 1].astype(np.float64), ny, nx, p, p, lam).ravel() for j in range(n)], 1)
    cr = torch.tensor(c0, dtype=torch.complex128, requires_grad=True)
    Ur = torch.from_numpy(A) @ cr
    lr = (Ur - torch.from_numpy(T.ravel())).abs().pow(2).sum()
    lr.backward()
    assert abs(loss.item() - lr.item()) / lr.item() < 1e-5
    assert rel_l2(c.grad.cpu().numpy(), cr.grad.numpy()) < TOL
