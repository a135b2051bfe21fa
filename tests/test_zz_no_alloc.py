"""hc_bin_tiles_noalloc (tile binning with no device allocation) against the
handle's own binning (hc_read_bins): bit-exact on two calls in a row, each
on a different state, so the second call also shows that the shared counters
left by the first are cleared.  Runs last so that it is exercised both after
the other tests and, run on its own, in a fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_TILES = 131072


def _case():
    from hemocell_gb300 import cases
    return cases.kolmogorov_mix(n=40, rbc_fraction=0.25, n_wbc=1, plt_per_rbc=0.2, wbc_triangles=1280, seed=3)


def _vertex_cells(case):
    return np.concatenate([np.full(xyz.shape[0], k, np.int32) for k, (_, xyz) in enumerate(case.cells)])


def _outputs(torch, ntiles, nvert, max_cells):
    dev = torch.device("cuda", 0)
    return dict(tile_offsets=torch.empty((ntiles + 1,), dtype=torch.int32, device=dev),
                tile_vertices=torch.empty((max(nvert, 1),), dtype=torch.int32, device=dev),
                tile_cell_offsets=torch.empty((ntiles + 1,), dtype=torch.int32, device=dev),
                tile_cells=torch.empty((max(max_cells, 1),), dtype=torch.int32, device=dev))


def _call(lib, torch, vtile, vcell, ntiles, max_cells, out=None, host=True):
    nvert = int(vtile.shape[0])
    if out is None:
        out = _outputs(torch, ntiles, nvert, max_cells)
    for v in out.values():
        v.fill_(-7)
    stream = torch.cuda.current_stream(vtile.device)
    rc = lib.hc_bin_tiles_noalloc(C.c_void_p(vtile.data_ptr()), C.c_void_p(vcell.data_ptr()), nvert, ntiles,
                                  C.c_void_p(out["tile_offsets"].data_ptr()),
                                  C.c_void_p(out["tile_vertices"].data_ptr()),
                                  C.c_void_p(out["tile_cell_offsets"].data_ptr()),
                                  C.c_void_p(out["tile_cells"].data_ptr()), max_cells,
                                  C.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.hc_last_error(None)
    stream.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()} if host else None


def _check_against(got, ref):
    nt = ref["tile_offsets"].shape[0] - 1
    assert np.array_equal(got["tile_offsets"], ref["tile_offsets"])
    assert np.array_equal(got["tile_vertices"][: ref["tile_offsets"][nt]], ref["tile_vertices"])
    assert np.array_equal(got["tile_cell_offsets"], ref["tile_cell_offsets"])
    assert np.array_equal(got["tile_cells"][: ref["tile_cell_offsets"][nt]], ref["tile_cells"])


def test_noalloc_binning_matches_handle_binning_twice(built):
    torch = pytest.importorskip("torch")
    from hemocell_gb300 import _lib as L
    lib = L.lib()
    dev = torch.device("cuda", 0)
    case = _case()
    hc = case.build(form=L.HC_FORM_MIXED_F32, launch=L.HC_LAUNCH_BATCHED, tile=(4, 4, 4))
    vcell = torch.from_numpy(_vertex_cells(case)).to(dev)
    V = int(vcell.shape[0])
    try:
        for call in range(2):
            hc.iterate(10 + 30 * call)          # a different state for each call
            ref = hc.read_bins()
            nt = ref["tile_offsets"].shape[0] - 1
            assert nt == 10 ** 3 and ref["tile_offsets"][nt] == V
            assert np.diff(ref["tile_cell_offsets"]).max() >= 2   # tiles shared by several cells
            vtile = torch.from_numpy(np.ascontiguousarray(ref["vertex_tile"], np.int32)).to(dev)
            got = _call(lib, torch, vtile, vcell, nt, V)
            _check_against(got, ref)

        # once set up, a call takes no device memory: the free amount is unchanged
        out = _outputs(torch, nt, V, V)
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info(dev)
        _call(lib, torch, vtile, vcell, nt, V, out=out, host=False)
        free1, _ = torch.cuda.mem_get_info(dev)
        assert free1 == free0
        _check_against({k: v.cpu().numpy() for k, v in out.items()}, ref)

        # tiles outside [0, ntiles) are left out like unbinned ones
        vt2 = vtile.clone()
        vt2[::7] = nt + 5
        host = vt2.cpu().numpy()
        got = _call(lib, torch, vt2, vcell, nt, V)
        keep = np.flatnonzero((host >= 0) & (host < nt))
        assert got["tile_offsets"][nt] == keep.size
        counts = np.bincount(host[keep], minlength=nt)
        assert np.array_equal(np.diff(got["tile_offsets"]), counts)
        order = np.lexsort((keep, host[keep]))
        assert np.array_equal(got["tile_vertices"][: keep.size], keep[order])
    finally:
        hc.close()


def test_noalloc_rejects_sizes_beyond_the_fixed_maximum(built):
    torch = pytest.importorskip("torch")
    from hemocell_gb300 import _lib as L
    lib = L.lib()
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    rc = lib.hc_bin_tiles_noalloc(p, p, 4, MAX_TILES + 1, p, p, p, p, 4, None)
    assert rc == L.HC_ERR_INVALID
    assert b"131072" in lib.hc_last_error(None)
    rc = lib.hc_bin_tiles_noalloc(p, p, 4, 0, p, p, p, p, 4, None)
    assert rc == L.HC_ERR_INVALID


def test_noalloc_crowded_tile_and_many_tiles(built):
    """More tiles than one scan block (5000 > 1024) and one tile holding 6000
    vertices (beyond the 2048 the shared-memory sort holds), against a numpy
    restatement of the lists: vertices ascending per tile, distinct cells per
    tile ascending (vertex ids grow with the cell id).  Called twice with
    different contents, as a second call also shows the counters cleared."""
    torch = pytest.importorskip("torch")
    from hemocell_gb300 import _lib as L
    lib = L.lib()
    dev = torch.device("cuda", 0)
    nt, V = 5000, 40000
    vcell_h = (np.arange(V) // 642).astype(np.int32)
    vcell = torch.from_numpy(vcell_h).to(dev)
    rng = np.random.default_rng(17)
    for call in range(2):
        vt = rng.integers(0, nt, V).astype(np.int32)
        crowd = rng.choice(V, 6000, replace=False)
        vt[crowd] = 17 + call
        vt[rng.choice(V, 50, replace=False)] = -1            # unbinned
        got = _call(lib, torch, torch.from_numpy(vt).to(dev), vcell, nt, V)
        keep = np.flatnonzero(vt >= 0)
        counts = np.bincount(vt[keep], minlength=nt)
        assert counts[17 + call] > 2048
        offs = np.concatenate([[0], np.cumsum(counts)])
        assert np.array_equal(got["tile_offsets"], offs)
        order = keep[np.lexsort((keep, vt[keep]))]
        assert np.array_equal(got["tile_vertices"][: keep.size], order)
        cells = [np.unique(vcell_h[order[offs[t]:offs[t + 1]]]) for t in range(nt)]
        coffs = np.concatenate([[0], np.cumsum([c.size for c in cells])])
        assert np.array_equal(got["tile_cell_offsets"], coffs)
        assert np.array_equal(got["tile_cells"][: coffs[-1]], np.concatenate(cells))
