"""Host-side logic on the CPU: setup utilities against the oracle, the
zodiax-style object model, layer keys, units, and the multi-rank partition."""

import os

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from oracle import dlux_oracle as O


def test_noll_map_matches_oracle():
    from dlux_gb300.utils import noll_indices
    for j in range(1, 300):
        assert noll_indices(j) == O.noll_indices(j)


def test_zernike_factors_match_oracle():
    from dlux_gb300.utils import zernike_factors
    for j in range(1, 40):
        c, k = zernike_factors(j)
        c0, k0 = O.zernike_factors(j)
        assert np.allclose(c, c0) and np.allclose(k, k0)


def test_zernike_basis_matches_oracle():
    from dlux_gb300.utils import zernike_basis
    coords = O.pixel_coords(64, 1.0)
    a = zernike_basis(range(1, 25), coords, 1.01, as_numpy=True)
    b = O.zernike_basis(range(1, 25), coords, 1.01)
    assert np.allclose(a, b, atol=1e-12)


def test_circular_aperture_matches_oracle():
    import dlux_gb300.utils as dlu
    T, B = dlu.circular_aperture(64, 1.0, oversample=3, secondary_diameter=0.1, spider_width=0.02,
                                 spider_angles=(0, 90, 180, 270), zernike_nolls=range(4, 10))
    T0, B0 = O.circular_aperture(64, 1.0, oversample=3, secondary_diameter=0.1, spider_width=0.02,
                                 spider_angles=(0, 90, 180, 270), zernike_nolls=list(range(4, 10)))
    assert np.allclose(T.cpu().numpy(), T0, atol=1e-6)
    assert np.allclose(B.cpu().numpy(), B0, atol=1e-5)


def test_units():
    import dlux_gb300.utils as dlu
    assert np.isclose(dlu.arcsec2rad(1.0), np.pi / 180 / 3600)
    assert np.isclose(dlu.rad2arcsec(dlu.arcsec2rad(0.02)), 0.02)
    assert np.isclose(dlu.unit_factor_to_rad("mas"), np.pi / 180 / 3600 / 1000)
    with pytest.raises(ValueError):
        dlu.unit_factor_to_rad("furlong")


def test_list2dictionary_keys():
    from dlux_gb300.helpers import list2dictionary

    class L1:
        pass

    d = list2dictionary([L1(), ("named", L1()), L1()], True)
    assert list(d) == ["L1_0", "named", "L1_1"]
    with pytest.raises(ValueError):
        list2dictionary([("has space", L1())], True)


def test_base_set_paths():
    from dlux_gb300.base import Base
    from collections import OrderedDict

    class Leaf(Base):
        def __init__(self):
            self.c = 1.0

    class Node(Base):
        def __init__(self):
            self.layers = OrderedDict(a=Leaf())

    n = Node()
    m = n.set("layers.a.c", 5.0)
    assert m.get("layers.a.c") == 5.0 and n.get("layers.a.c") == 1.0
    assert n.multiply("layers.a.c", 3.0).layers["a"].c == 3.0


def test_fusion_description_of_layers():
    """The fused path's pupil description follows dLux's layer semantics."""
    import dlux_gb300 as dl
    from dlux_gb300.layers.optical_layers import PupilAccumulator
    T = torch.ones((8, 8))
    acc = PupilAccumulator(8)
    for layer in [dl.TransmissiveLayer(T, normalise=True), dl.AberratedLayer(opd=torch.zeros(8, 8)),
                  dl.Tilt([1e-7, 0.0])]:
        layer.fuse(acc)
    assert acc.normalised and len(acc.pre) == 1 and not acc.post
    assert acc.tilt.tolist() == [1e-7, 0.0] and len(acc.opd_static) == 1
    with pytest.raises(dl.layers.optical_layers.NotFusable):
        dl.MFT(16, 1e-7).fuse(acc)


def test_shard_range_covers_units():
    from dlux_gb300.partition import shard_range
    for n in (1, 5, 64, 1024):
        for world in (1, 2, 3, 8):
            blocks = [shard_range(n, world, r) for r in range(world)]
            assert blocks[0][0] == 0 and blocks[-1][1] == n
            assert all(b[1] == nb[0] for b, nb in zip(blocks, blocks[1:]))
            sizes = [b[1] - b[0] for b in blocks]
            assert max(sizes) - min(sizes) <= 1


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from dlux_gb300.partition import reduce_partial, shard_units
    T, B = O.circular_aperture(32, 1.0, oversample=3, secondary_diameter=0.1,
                               zernike_nolls=list(range(4, 8)))
    opd = O.eval_basis(B, np.array([20e-9, -10e-9, 5e-9, 30e-9]))
    wls = np.linspace(0.8e-6, 1.2e-6, 7)
    w = np.linspace(1, 2, 7) / np.linspace(1, 2, 7).sum()
    mine = shard_units(np.arange(7), world, rank)
    part = O.poly_psf(T, opd, wls[mine], w[mine], 1.0, 16, float(O.arcsec2rad(0.05)))
    t = torch.as_tensor(part)
    reduce_partial(t)
    if rank == 0:
        np.save(out_path, t.numpy())
    dist.destroy_process_group()


def test_wavelength_partition_with_gloo(tmp_path):
    """world_size 2: each rank sums its wavelength block; one all-reduce gives the full PSF."""
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    out = str(tmp_path / "psf.npy")
    mp.start_processes(_rank_main, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    T, B = O.circular_aperture(32, 1.0, oversample=3, secondary_diameter=0.1,
                               zernike_nolls=list(range(4, 8)))
    opd = O.eval_basis(B, np.array([20e-9, -10e-9, 5e-9, 30e-9]))
    wls = np.linspace(0.8e-6, 1.2e-6, 7)
    w = np.linspace(1, 2, 7) / np.linspace(1, 2, 7).sum()
    full = O.poly_psf(T, opd, wls, w, 1.0, 16, float(O.arcsec2rad(0.05)))
    assert np.allclose(np.load(out), full, rtol=1e-12, atol=0)
