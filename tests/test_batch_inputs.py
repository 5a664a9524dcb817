"""The seeded ensemble inputs (opensbli_gb300.batch.tgv_ensemble) on CPU: deterministic sizes and
schemes, band-limited perturbations of the stated RMS amplitude, positive CFL time steps."""
import torch

from opensbli_gb300.batch import band_limited_field, tgv_ensemble


def test_band_limited_field_spectrum_and_amplitude():
    f = band_limited_field(24, 4, seed=5, device="cpu", amplitude=1e-2)
    assert f.shape == (3, 24, 24, 24)
    for c in range(3):
        assert abs(float(f[c].pow(2).mean().sqrt()) - 1e-2) < 1e-12
        F = torch.fft.fftn(f[c])
        k = torch.fft.fftfreq(24, d=1.0 / 24)
        KZ, KY, KX = torch.meshgrid(k, k, k, indexing="ij")
        outside = (KX ** 2 + KY ** 2 + KZ ** 2) > 16
        assert float(F[outside].abs().max()) < 1e-12 * float(F.abs().max())
    g = band_limited_field(24, 4, seed=5, device="cpu", amplitude=1e-2)
    assert torch.equal(f, g)


def test_tgv_ensemble_is_seeded():
    a = tgv_ensemble(count=8, sizes=(16, 24), seed=1, device="cpu")
    b = tgv_ensemble(count=8, sizes=(16, 24), seed=1, device="cpu")
    assert [p.n for p in a[0]] == [p.n for p in b[0]]
    assert [p.conv for p in a[0]] == [p.conv for p in b[0]]
    assert all(torch.equal(x, y) for x, y in zip(a[1], b[1]))
    assert all(dt > 0 for dt in a[2])
    assert {p.n[0] for p in a[0]} <= {16, 24}
