"""The benchmark's own configuration at full size against the FP64 oracle.

512^2 pupil (1 m, 10% obscuration, four 1 cm spiders), 21 Zernikes
N(0, 30 nm), 64 wavelengths on 0.8-1.2 um with Dirichlet(1) weights, MFT to
512^2 at 4x oversampling of 0.02"/px, 4 x 4 sum downsample to 128^2, and the
gradient of sum(R * image) w.r.t. the coefficients. The inputs are those of
bench.py, the step is the public API the benchmark times, and both forms must
be within 1e-5 (relative L2) of the FP64 restatement: the split-BF16 form is
the benchmarked one, the FP32 form its reference on the GPU.
"""

import numpy as np
import pytest
import torch

from oracle import dlux_oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("variant", ["split_bf16", "fp32"])
def test_headline_configuration_matches_fp64_oracle(cuda, variant):
    import bench
    import dlux_gb300 as dl

    coeffs, wls, weights, R = bench.make_inputs()
    T, B = O.circular_aperture(bench.N_PUPIL, 1.0, oversample=5, secondary_diameter=0.1,
                               spider_width=0.01, spider_angles=(0, 90, 180, 270),
                               zernike_nolls=bench.NOLLS)
    ps_out = float(O.arcsec2rad(bench.PSF_PIXEL_SCALE / bench.OVERSAMPLE))
    opd = np.tensordot(B, coeffs, axes=(0, 0))
    psf = O.poly_psf(T, opd, wls, weights, 1.0, bench.N_FOCAL, ps_out)
    img_ref = O.downsample(psf, bench.OVERSAMPLE, mean=False)
    Teff = T / np.sqrt((T ** 2).sum())
    G = np.kron(R, np.ones((bench.OVERSAMPLE, bench.OVERSAMPLE)))
    g = O.poly_psf_grad(Teff, opd, wls, weights, 1.0, bench.N_FOCAL, ps_out, G)
    gc_ref = np.tensordot(B, g["g_opd"], axes=((1, 2), (0, 1)))

    dl.set_variant(variant)
    try:
        f32 = dict(dtype=torch.float32, device="cuda")
        c = torch.as_tensor(coeffs, **f32)
        optics = dl.AngularOpticalSystem(
            bench.N_PUPIL, 1.0,
            [dl.TransmissiveLayer(torch.as_tensor(T, **f32), normalise=True),
             dl.BasisLayer(torch.as_tensor(B, **f32), c)],
            bench.N_FOCAL // bench.OVERSAMPLE, bench.PSF_PIXEL_SCALE, bench.OVERSAMPLE)
        detector = dl.LayeredDetector([dl.Downsample(bench.OVERSAMPLE)])
        _, gc, img = bench.step(optics, detector, wls, torch.as_tensor(weights, **f32),
                                torch.as_tensor(R, **f32), c)
        torch.cuda.synchronize()
    finally:
        dl.set_variant(None)
    e_img = np.linalg.norm(img.cpu().numpy() - img_ref) / np.linalg.norm(img_ref)
    e_g = np.linalg.norm(gc.cpu().numpy() - gc_ref) / np.linalg.norm(gc_ref)
    print(f"{variant}: image rel L2 {e_img:.2e}, coefficient-gradient rel L2 {e_g:.2e}")
    assert e_img < 1e-5 and e_g < 1e-5
