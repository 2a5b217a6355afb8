"""voce_mesh_voronoi: the periodic Voronoi microstructure computed on the GPU
equals the host generator's, voxel for voxel (labels, grains, orientations),
on an anisotropic grid and on the 64^3 / 125-grain mesh of the parity
fixture (whose digest it must reproduce)."""
import numpy as np
import pytest

from voce_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _seeds(n_grains, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    seeds = rng.random((n_grains, 3))
    return seeds, synth.so3_uniform_bunge(rng, n_grains)


def test_voronoi_matches_host_generator_anisotropic(voce_lib):
    dims = (24, 20, 16)
    seeds, eul_g = _seeds(37, 91)
    want = synth.voronoi_mesh_box(dims, 37, 91)
    eul, grain, phase = capi.mesh_voronoi(dims, seeds, eul_g)
    assert np.array_equal(grain, want.grain)
    assert np.array_equal(eul, want.euler_deg) and (phase == 1).all()


def test_voronoi_reproduces_the_parity_mesh(voce_lib):
    want = synth.config2(1).mesh          # 64^3, 125 grains, seed 2
    seeds, eul_g = _seeds(125, 2)
    eul, grain, phase = capi.mesh_voronoi(want.dims, seeds, eul_g)
    got = synth.Mesh(want.dims, eul, grain, phase)
    assert got.digest() == want.digest()


def test_voronoi_many_seeds_more_than_one_tile(voce_lib):
    # 2500 seeds: the kernel walks them in shared-memory tiles of 1024
    dims = (20, 20, 20)
    seeds, eul_g = _seeds(2500, 93)
    want = synth.voronoi_mesh_box(dims, 2500, 93)
    eul, grain, phase = capi.mesh_voronoi(dims, seeds, eul_g)
    assert np.array_equal(grain, want.grain)
