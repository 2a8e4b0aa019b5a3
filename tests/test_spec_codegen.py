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
