"""sph_count_pairs_noalloc: the pair counter for callers that cannot let the library
allocate device memory (their memory belongs to another framework's pool, or they
must avoid the device-wide synchronisation cudaMalloc/cudaFree can cause).

The caller owns the device buffers (allocated here with torch, as such a caller
would with its own allocator) and the stream; the result must equal sph_count_pairs
of a regular handle exactly (integer counts), on two calls in a row, including a
second scene of another size that reuses the shared scratch array.  This file runs
last so that a failure here stops a `-x` run only after every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def handle_counts(pkg, scene, sub=0):
    with pkg.Simulation(scene.params(cell_subdivision=sub), scene.n_fluid, scene.n_wall) as sim:
        for w in scene.walls:
            sim.upload_walls(w)
        sim.upload_fluid(scene.fluid)
        return sim.count_pairs()


def noalloc_counts(lib, scene, torch, sub=0):
    x = torch.from_numpy(np.ascontiguousarray(scene.fluid.x_vec_)).cuda()
    wx = torch.from_numpy(np.ascontiguousarray(np.concatenate([w.x_vec_ for w in scene.walls]))).cuda()
    out = torch.full((2,), -1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    prm = scene.params(cell_subdivision=sub)
    rc = lib.sph_count_pairs_noalloc(C.byref(prm), len(x), C.c_void_p(x.data_ptr()), len(wx),
                                     C.c_void_p(wx.data_ptr()), C.c_void_p(out.data_ptr()),
                                     C.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.sph_last_error(None)
    stream.synchronize()
    return tuple(int(v) for v in out.cpu())


def test_noalloc_pair_counts_match_handle(pkg):
    torch = pytest.importorskip("torch")
    from ethersph_gb300 import _abi, scenes
    lib = _abi.load_library()
    big = scenes.dam_break_2d(dx=0.02)            # 5,000 fluid + 1,518 walls
    small = scenes.natural_convection_2d(n=64)    # 4,096 fluid + 780 walls, other grid
    expect_big = handle_counts(pkg, big)
    expect_small = handle_counts(pkg, small)
    assert expect_big[0] > 0 and expect_big[1] > 0
    # two calls in a row on the same input, then a different scene over the same scratch
    assert noalloc_counts(lib, big, torch) == expect_big
    assert noalloc_counts(lib, big, torch) == expect_big
    assert noalloc_counts(lib, small, torch) == expect_small
    assert noalloc_counts(lib, big, torch) == expect_big


def test_noalloc_other_grids_match_handle(pkg):
    # the 3D hash and walk, the periodic x wrap of the pair distance, and one cell per
    # r_cut (reach 1) instead of the default two, each against a regular handle
    torch = pytest.importorskip("torch")
    from ethersph_gb300 import _abi, scenes
    lib = _abi.load_library()
    cases = [(scenes.dam_break_3d(dx=0.05, tank=(0.6, 0.3, 0.4), column=(0.2, 0.2, 0.3)), 0),
             (scenes.poiseuille_periodic_2d(n_across=16), 0),
             (scenes.dam_break_2d(dx=0.04), 1)]
    for s, sub in cases:
        expect = handle_counts(pkg, s, sub)
        assert expect[0] > 0
        assert noalloc_counts(lib, s, torch, sub) == expect, s.name
        assert noalloc_counts(lib, s, torch, sub) == expect, s.name


def test_noalloc_call_allocates_no_device_memory(pkg):
    # after a first call (which looks up the scratch array's address), a call leaves the
    # device's free memory exactly as it was
    torch = pytest.importorskip("torch")
    from ethersph_gb300 import _abi, scenes
    lib = _abi.load_library()
    s = scenes.dam_break_2d(dx=0.02)
    x = torch.from_numpy(np.ascontiguousarray(s.fluid.x_vec_)).cuda()
    wx = torch.from_numpy(np.ascontiguousarray(s.walls[0].x_vec_)).cuda()
    out = torch.zeros(2, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    prm = s.params()

    def call():
        rc = lib.sph_count_pairs_noalloc(C.byref(prm), len(x), C.c_void_p(x.data_ptr()), len(wx),
                                         C.c_void_p(wx.data_ptr()), C.c_void_p(out.data_ptr()),
                                         C.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.sph_last_error(None)
        stream.synchronize()

    call()
    free_before = torch.cuda.mem_get_info()[0]
    call()
    assert torch.cuda.mem_get_info()[0] == free_before


def test_noalloc_rejects_sizes_beyond_the_limit(pkg):
    torch = pytest.importorskip("torch")
    from ethersph_gb300 import _abi, scenes
    lib = _abi.load_library()
    s = scenes.dam_break_2d(dx=0.05)
    prm = s.params()
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = torch.zeros(2, dtype=torch.int64, device="cuda")
    rc = lib.sph_count_pairs_noalloc(C.byref(prm), 262145, C.c_void_p(dummy.data_ptr()), 0, None,
                                     C.c_void_p(out.data_ptr()), None)
    assert rc == 1
    assert b"262144" in lib.sph_last_error(None)
    # a grid with more cells than the scratch holds
    prm.domain_hi[0] = prm.domain_lo[0] + 1e4 * prm.influence_radius
    prm.domain_hi[1] = prm.domain_lo[1] + 100 * prm.influence_radius
    rc = lib.sph_count_pairs_noalloc(C.byref(prm), 1, C.c_void_p(dummy.data_ptr()), 0, None,
                                     C.c_void_p(out.data_ptr()), None)
    assert rc == 1
    assert b"cells" in lib.sph_last_error(None)
