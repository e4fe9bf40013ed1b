"""The spectral extension's colour science, pinned on the CPU: the analytic
CIE 1931 fit integrates to the reference's own Y normalisation
(kCIENormalizationY = 1 / 106.8569, Core/Spectrum.h:286) and has the equal
energy white point of the tabulated functions; grey RGB upsamples to a flat
spectrum; the white balance maps a flat spectrum to RGB (1, 1, 1)."""
import numpy as np

import oracle

M = np.array([[3.2404542, -1.5371385, -0.4985314], [-0.9692660, 1.8760108, 0.0415560],
              [0.0556434, -0.2040259, 1.0572252]])


def test_cmf_integrals_match_cie_normalisation():
    lam = np.arange(360.0, 830.0, 0.05, dtype=np.float32) + 0.025
    xyz = oracle.spectral_cmf(lam).astype(np.float64) * 0.05
    ix, iy, iz = xyz.sum(0)
    assert abs(iy - 106.8569131841719) / 106.8569131841719 < 2e-3
    assert abs(ix - iy) / iy < 3e-3 and abs(iz - iy) / iy < 3e-3
    y = oracle.spectral_cmf(np.float32([555.0]))[0, 1]
    assert abs(y - 1.0) < 0.01


def test_grey_is_flat_and_white_balance():
    lam = np.linspace(360, 829, 200).astype(np.float32)
    for a in (0.2, 0.5, 0.8):
        s = oracle.spectral_upsample(np.full((len(lam), 3), a, np.float32), lam)
        np.testing.assert_allclose(s, a, rtol=2e-6)
    wb = oracle.spectral_white_balance().astype(np.float64)
    lam = np.arange(360.0, 830.0, 0.1, dtype=np.float32) + 0.05
    xyz = oracle.spectral_cmf(lam).astype(np.float64).sum(0) * 0.1
    np.testing.assert_allclose(M @ xyz * wb, 1.0, rtol=1e-3)
