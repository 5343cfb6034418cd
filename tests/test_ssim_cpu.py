"""CPU pin of the SSIM oracle: oracle.ssim_map / ssim_backward / l1_dssim against
tests/golden/ssim_golden.npz, which holds the reference's own SSIM and training
loss (3DGS/utils/loss_utils.py ssim and l1_loss) and their autograd gradients
in FP64.  The reference rounds its window to float32 before use, the oracle
keeps it in FP64: values agree to 1e-7, gradients to 1e-6 of their largest
entry."""
from pathlib import Path

import numpy as np

import oracle

GOLD = np.load(Path(__file__).resolve().parent / "golden" / "ssim_golden.npz")


def _rel(a, b):
    return float(np.abs(a - b).max()) / max(float(np.abs(b).max()), 1e-30)


def test_ssim_window_is_the_normalised_gaussian():
    w = oracle.ssim_window()
    assert w.shape == (11,) and abs(w.sum() - 1.0) < 1e-15 and np.allclose(w, w[::-1])
    assert np.argmax(w) == 5


def test_ssim_and_gradient_match_reference():
    for k in (0, 1):
        img, gt = GOLD[f"img{k}"], GOLD[f"gt{k}"]
        m, a, b, c = oracle.ssim_map(img, gt)
        per_image = m.reshape(m.shape[0], -1).mean(1)
        assert np.abs(per_image - GOLD[f"ssim{k}"]).max() < 1e-7
        g = oracle.ssim_backward(img, gt, np.full_like(m, 1.0 / m[0].size), a, b, c)
        assert _rel(g, GOLD[f"grad_ssim{k}"]) < 1e-6


def test_training_loss_and_gradient_match_reference():
    lam = float(GOLD["lam"])
    for k in (0, 1):
        loss, _, g = oracle.l1_dssim(GOLD[f"img{k}"], GOLD[f"gt{k}"], lam)
        assert abs(loss - float(GOLD[f"loss{k}"])) < 1e-7
        assert _rel(g, GOLD[f"grad_loss{k}"]) < 1e-6


def test_ssim_partials_match_finite_differences():
    """dm/dmu1, dm/dE[x^2], dm/dE[xy] of the oracle against central differences of m."""
    rng = np.random.default_rng(3)
    mo = rng.uniform(0.1, 0.9, size=(5, 64))
    mo[2] = mo[0] ** 2 + rng.uniform(0.001, 0.05, 64)   # E[x^2] >= mu1^2
    mo[3] = mo[1] ** 2 + rng.uniform(0.001, 0.05, 64)
    mo[4] = mo[0] * mo[1] + rng.uniform(-0.01, 0.01, 64)
    C1, C2 = 0.01 ** 2, 0.03 ** 2

    def m_of(mu1, mu2, e11, e22, e12):
        C = 2 * mu1 * mu2 + C1
        D = 2 * (e12 - mu1 * mu2) + C2
        A = mu1 ** 2 + mu2 ** 2 + C1
        B = (e11 - mu1 ** 2) + (e22 - mu2 ** 2) + C2
        return C * D / (A * B)

    mu1, mu2, e11, e22, e12 = mo
    _, d_mu1, d_e11, d_e12 = oracle.ssim_from_moments(mu1, mu2, e11, e22, e12, C1, C2)
    h = 1e-6
    fd_mu1 = (m_of(mu1 + h, mu2, e11, e22, e12) - m_of(mu1 - h, mu2, e11, e22, e12)) / (2 * h)
    fd_e11 = (m_of(mu1, mu2, e11 + h, e22, e12) - m_of(mu1, mu2, e11 - h, e22, e12)) / (2 * h)
    fd_e12 = (m_of(mu1, mu2, e11, e22, e12 + h) - m_of(mu1, mu2, e11, e22, e12 - h)) / (2 * h)
    assert _rel(d_mu1, fd_mu1) < 1e-6
    assert _rel(d_e11, fd_e11) < 1e-6
    assert _rel(d_e12, fd_e12) < 1e-6
