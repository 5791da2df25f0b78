"""The parallel FP64 full step of bench.py's reference arm (oracle/cpu_step.py
FullStep: advection on haloed z-slabs, resamplings on output boxes, raymarch
on (camera, row band) windows with per-camera reduction of the partial sums
before the reference normalisation) equals the serial FP64 step oracle."""
import numpy as np
import pytest

from scene_utils import rel_l2


@pytest.mark.parametrize('config,workers', [('tiny', 2), ('cfg1', 3)])
def test_full_step_equals_serial_oracle(config, workers):
    from oracle import cpu_step as CS
    from oracle import step as OS
    sc, fc, d, vel, target = CS.scene_arrays(config)
    sc2 = dict(sc)
    sc2['falloff_col'] = fc
    loss, _, grads = OS.step(sc2, d, *vel, target)
    with CS.FullStep(config, workers=workers) as fs:
        loss2, seconds = fs.step()
        got = fs.gradients()
    assert seconds > 0
    assert abs(loss2 - loss) <= 1e-12 * abs(loss)
    for a, b in zip(got, grads):
        assert rel_l2(a, b) <= 1e-12
