"""CPU oracle for the dLux diffraction hot path.

TEST INFRASTRUCTURE ONLY. Nothing in the shipped package imports this module:
only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may use it, and only as the checker.

``dlux_oracle`` restates, in NumPy, the arithmetic of dLux v0.16.0 on the
diffraction hot path (MFT, FFT propagation, Zernike-basis OPD to phasor,
polychromatic |E|^2 sum, detector downsample) and its reverse-mode gradient.
Every function takes a ``precision`` switch:

* ``"f64"`` -- the FP64 oracle every error is measured against;
* ``"c64"`` -- a float32/complex64 mimic of dLux's own op order (dLux never
  enables JAX x64), which stands in for dLux's CPU path.

Parity status: dLux's tests pin only structural facts and a handful of known
answers (Noll indices, FFT round trip, MFT shift equivalence, fft_spec offsets,
ramp conjugacy, eval_basis == tensordot, downsample shapes). Those are checked
against this oracle in ``tests/test_oracle.py``. PSF/gradient *values* are not
pinned by any reference golden vector (the reference cannot be imported here:
jax, equinox and zodiax are absent), so value parity rests on this restatement
plus physics known-answer tests (Parseval, MFT == FFT at matched sampling,
adjoint identity, central finite differences).
"""
