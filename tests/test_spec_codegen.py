"""Topology-specialised kernels: code generation and NVRTC compilation for
sm_103a run on the CPU (no device needed)."""
import pytest

from spicier_gb300 import abi, configs
from spicier_gb300.api import specialized_source


@pytest.mark.parametrize("make", [configs.cs_nmos_amp, configs.miller_opamp, configs.bjt_diode_bias])
@pytest.mark.parametrize("prec", [abi.SP_PREC_MIXED, abi.SP_PREC_FP64])
def test_generated_kernel_compiles(product_lib, make, prec):
    c = make()
    src, nnz = specialized_source(c, prec, compile=True)
    assert "spec_newton" in src
    assert c.n <= nnz <= c.n * c.n


def test_opamp_factorisation_is_sparse(product_lib):
    _, nnz = specialized_source(configs.miller_opamp(), abi.SP_PREC_MIXED)
    assert nnz < 0.5 * 12 * 12  # structural nonzeros + fill of the static order


def test_structurally_singular_circuit_is_rejected(product_lib):
    from spicier_gb300 import Circuit, SpicierError
    c = Circuit("floating")
    c.Cap("C1", "a", "0", 1e-12)  # node a has no DC path: empty column
    c.R("R1", "b", "0", 1.0)
    with pytest.raises(SpicierError):
        specialized_source(c, abi.SP_PREC_MIXED)


def test_double_float_parameters_mode(product_lib):
    """R/C/L/V/I/MOS circuits in mixed precision: double-float state and
    residual, constants computed from the drawn parameters (fixed ones as
    exact literals), FP64 constants written only for listed samples; circuits
    with diodes or BJTs keep the FP64 residual and the derived constants."""
    src, _ = specialized_source(configs.miller_opamp(), abi.SP_PREC_MIXED)
    assert "spx_df X[" in src and "a.lp + (u64)" in src and "a.dvo[" in src
    assert "a.dv + s" not in src
    assert "0x" in src  # fixed parameters as hexadecimal literals
    src64, _ = specialized_source(configs.miller_opamp(), abi.SP_PREC_FP64)
    assert "spx_df X[" not in src64 and "a.dv + s" in src64
    srcb, _ = specialized_source(configs.bjt_diode_bias(), abi.SP_PREC_MIXED)
    assert "spx_df X[" not in srcb and "a.dv + s" in srcb
