"""ast_get_phase_clocks: per-phase SM cycle counters of the persistent FP32
kernel, compiled in only by a profiling build (AST_PHASE_CLOCKS=1)."""
import os

import pytest

from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import problems, solver


@pytest.mark.gpu
def test_phase_clocks_unsupported_in_product_build():
    # the per-phase cycle counters exist only in a profiling build
    # (AST_PHASE_CLOCKS=1 at build time); the product build refuses the call
    if os.environ.get("AST_PHASE_CLOCKS", "0") == "1":
        pytest.skip("profiling build")
    cfg = problems.blast_config(64, 32, flux=A.FLUX_HLL, precision=A.PREC_FP32)
    with solver.Solver(cfg) as S:
        with pytest.raises(solver.AstError) as e:
            S.phase_clocks()
        assert e.value.code == A.AST_ERR_UNSUPPORTED
