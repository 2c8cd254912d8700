"""The entry module's smoke run as a GPU test: one small frame (RebuildTopology ->
UpdateAtlas -> InsertPointsSubcell -> GatherDensity -> UpdateApron) on cuda:0 through
the C ABI, its node pools, subcell-list length and atlas checked against the oracle."""
import pytest


@pytest.mark.gpu
def test_smoke(gpu_lib):
    import __graft_entry__

    __graft_entry__.smoke()
