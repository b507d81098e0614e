"""What the trained warm-start network (curvedspacevertexmodel_gb300/data/warm_start_n20k.npz,
trained on the GPU by the library's kernels with `python -m curvedspacevertexmodel_gb300.warm_start
train`) gains over the method without it, on a held-out instance: the network's displacement
lowers the energy of the start state, and FIRE from there reaches the same force tolerance."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def svm(svm_lib):
    if svm_lib.device_count() < 1:
        pytest.fail("no CUDA device: the GPU tests need a GB300")
    return svm_lib


def test_warm_start_lowers_the_energy_and_fire_converges(svm):
    from curvedspacevertexmodel_gb300 import warm_start as ws
    net = ws.load(os.path.join(os.path.dirname(svm.__file__), "data", "warm_start_n20k.npz"))
    r = ws.compare(net, 5000, 3.65, 777)
    print(r)
    assert r["plain_max_force"] < 1e-9 and r["warm_max_force"] < 1e-9
    # the untrained method (plain FIRE from the start state) begins from the start's energy; the
    # network's step lowers it
    assert r["energy_after_warm_start"] < 0.95 * r["energy_start"]
    assert r["fallback"] is None
    # both end in minima of the same model; they may be different local minima (here the warm one
    # is a few percent lower), and the warm one is not worse by more than a few percent
    assert r["energy_per_cell_warm"] < 1.05 * r["energy_per_cell_plain"]
