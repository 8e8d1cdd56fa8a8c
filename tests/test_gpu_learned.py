"""Learned GMRES preconditioner: the GPU forward and backward kernels of the U-Net against
the CPU oracle (oracle/unet_oracle.py, float64 with the same BF16-rounded weights), and the
iterations the trained network saves on the pressure solves of a cylinder case (GMRES still
iterates to the reference's true-residual tolerance, so the flow fields are unchanged)."""
import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu


def test_unet_forward_and_gradients_match_oracle():
    torch = pytest.importorskip('torch')
    import unet_oracle as uo
    learned = load_package().learned
    wts = learned.UNetWeights(seed=3)
    assert wts.count() == 253872 + 465
    B, H, W = 2, 16, 24
    rng = np.random.default_rng(5)
    x = rng.standard_normal((B, 2, H, W)).astype(np.float32)
    net = learned.UNet(B, H, W)
    y = net.forward(wts, torch.from_numpy(x).cuda())
    torch.cuda.synchronize()
    ws = [w.to(torch.float32).cpu().numpy().astype(np.float64) for w in wts.w16]  # the BF16 values
    bs = [b.detach().cpu().numpy().astype(np.float64) for b in wts.b]
    y_ref, saved = uo.forward(x.astype(np.float64), ws, bs)
    assert np.max(np.abs(y.cpu().numpy() - y_ref)) < 1e-4 * np.max(np.abs(y_ref))
    dy = rng.standard_normal(y_ref.shape).astype(np.float32)
    dw, db = net.backward(wts, torch.from_numpy(dy).cuda())
    torch.cuda.synchronize()
    dws, dbs = uo.backward(saved, ws, dy.astype(np.float64))
    for k in range(12):
        g, r = dw[k].cpu().numpy(), dws[k]
        assert np.max(np.abs(g - r)) < 1e-3 * max(np.max(np.abs(r)), 1e-12), k
        g, r = db[k].cpu().numpy(), dbs[k]
        assert np.max(np.abs(g - r)) < 1e-3 * max(np.max(np.abs(r)), 1e-12), k
    net.close()


def test_learned_preconditioner_on_held_out_solves():
    """Trains the network on the solver's own pressure solves, then runs held-out solves of the
    same case with and without it.  GMRES iterates to the same true-residual tolerance either
    way, so the answers agree; the iteration counts and the network's held-out error are the
    measured gain (printed, and bounded below so that the network never costs more than one
    iteration per solve)."""
    torch = pytest.importorskip('torch')
    pkg = load_package()
    learned = pkg.learned
    kw = dict(nx=96, ny=48, Lx=9.6, Ly=4.8, D=1.0, xc=2.4, yc=2.4, nu=0.01, verbose=False,
              pressure_solver='iterative')
    s = pkg.MAC_CylinderFlow(**kw)
    rhs, sol = learned.record_pressure_pairs(s, 40, 0.002)
    assert rhs.shape[0] >= 60
    # train on the earlier solves, hold out the last four
    x, y, mask = learned.training_set(s, rhs[:-4], sol[:-4])
    xh, yh, _ = learned.training_set(s, rhs[-4:], sol[-4:])
    wts = learned.UNetWeights(seed=1)
    hist = learned.train(wts, x, y, mask, epochs=1500, lr=2e-3, batch=4)
    assert hist[-1] < 0.5 * hist[0]
    err = learned.relative_error(wts, xh, yh, mask)
    its_plain, its_learned = [], []
    for b in rhs[-4:].cpu().numpy():
        b = b.reshape(-1)[s.gg.pi]
        x0 = s.gg.pressure_solve(b)
        its_plain.append(s.gg.pressure_inverse_info['last_solve']['iterations'])
        pc = learned.LearnedPreconditioner(s, wts)
        x1 = s.gg.pressure_solve(b)
        its_learned.append(s.gg.pressure_inverse_info['last_solve']['iterations'])
        pc.detach()
        assert np.max(np.abs(x1 - x0)) < 1e-8 * max(1.0, np.max(np.abs(x0)))
    print(f'held-out relative error of the network: {err}; GMRES iterations plain {its_plain}, '
          f'with the network {its_learned}; final training loss / first: {hist[-1] / hist[0]:.3g}')
    assert all(l <= p + 1 for p, l in zip(its_plain, its_learned)), (its_plain, its_learned)
