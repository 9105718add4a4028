"""Without a CUDA device the product path refuses to run: no CPU fallback
(the oracle is test infrastructure only).  Skipped where a GPU is present."""
import pytest
import torch

from lbm_gb300.apps import cavity


@pytest.mark.skipif(torch.cuda.is_available(), reason="a CUDA device is present")
def test_lattice_refuses_to_run_without_a_gpu():
    import lbm_gb300
    app = cavity()
    app.L_lbm = 16
    app.compute_lbm_parameters()
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        lbm_gb300.lattice(app)

