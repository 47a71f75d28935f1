"""GPU test of gbsw_calibrate, the measured roofline of the passes.

The cell probes' throughput is timed with CUDA events; it must be positive and
stay below what an SM can issue at any SM clock up to 2.2 GHz.  A dual cell
pair is 6.5 ops, all on the integer ALU pipe, which takes a warp instruction
every other cycle per SM sub-partition (64 lane-ops per clock per SM).  An
int32 pass cell is 6.5 ops, some of which issue to other pipes, so it is
bounded by the issue rate (128 lane-ops per clock per SM); the int32 cell probe
is at least 3 ops."""
import pytest

pytestmark = pytest.mark.gpu


def test_calibration_bounds(built):
    c = built.calibrate(0)
    assert c["sms"] > 0
    alu_per_s = c["sms"] * 64 * 2.2e9
    issue_per_s = 2 * alu_per_s
    assert 0 < c["cell_dual_gcups"] * 1e9 < alu_per_s / 3.25
    assert 0 < c["cell_dpx_gcups"] * 1e9 < issue_per_s / 3
    assert 0 < c["cell_int32_gcups"] * 1e9 < issue_per_s / 6.5
    # per-tick rates are reported beside them; clock64 ticks per microsecond > 0
    assert c["sm_mhz"] > 0 and c["cell_dual"] > 0
