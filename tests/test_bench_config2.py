"""The reference arm of bench.py takes config 2's compatibility shift from a
recorded constant; it belongs to one geometry and right-hand side.  A shift
that no longer fits leaves a residual floor of about 51 times its error and
stalls every reference solve, so the recorded inputs are pinned here."""
import bench


def test_config2_shift_belongs_to_the_current_inputs():
    assert bench.config2_digest() == bench.CONFIG2_DIGEST, (
        "the config-2 geometry or right-hand side changed: recompute CONFIG2_SHIFT "
        "(problem.compatibility_shift with plateau solves) and CONFIG2_DIGEST in bench.py")
