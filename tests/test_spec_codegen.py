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


def test_linear_warm_start_launch_parameter_and_cold_restart(product_lib):
    """The double-float kernel carries the learned linear term's launch-parameter
    form (SpecLin: weights for every drawn slot the elements read, in ascending
    slot order, summed with constant-bank operands) beside the form read from
    memory; every generated kernel restarts a missed warm start from the nodeset
    in the same lane, with the full iteration limit."""
    src, _ = specialized_source(configs.miller_opamp(), abi.SP_PREC_MIXED)
    assert "struct SpecLin" in src and "spec_newton(SpecArgs a, SpecLin lk)" in src
    assert "if (lk.on) {" in src and "if (a.lw && !lk.on) {" in src
    # 17 drawn slots read by the op-amp's elements: 17 x 12 weights, 17 means, 12
    # outputs; the sample set-up appears twice (first sample, then each next one)
    assert "float w[233]" in src and src.count("if ((lk.mask >> ") == 2 * 17
    slots = [int(line.split("pf")[1].split(" ")[0]) for line in src.splitlines()
             if line.strip().startswith("const float v = pf")]
    assert slots[:17] == sorted(slots[:17]) and slots[17:] == slots[:17] and len(set(slots)) == 17
    for make, prec in ((configs.miller_opamp, abi.SP_PREC_FP64), (configs.bjt_diode_bias, abi.SP_PREC_MIXED)):
        s, _ = specialized_source(make(), prec)
        assert "if (lk.on) {" not in s  # only the double-float kernel takes the parameter form
        assert "spx_itlim = a.cold_max_it" in s
    assert "spx_itlim = a.cold_max_it" in src
