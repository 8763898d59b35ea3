"""The FP32 throughput probe behind the FP32 roofline: a plausible GB300 rate with scalar and with
packed f32x2 FMAs (152 SMs x 128 FP32 lanes x 2 flops at 1-2.1 GHz is 39-81 TFLOP/s nominal for
scalar FMAs) and argument checks on the host."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_fp32_peak_probe():
    import pfm
    torch.cuda.set_device(0)
    for packed in (False, True):
        rate = pfm.measure_fp32_peak(blocks_per_sm=4, iters=8192, reps=2, packed=packed)
        assert 20.0 < rate < 250.0, (packed, rate)


def test_fp32_peak_probe_rejects_bad_arguments():
    import pfm
    with pytest.raises(pfm.PfmError):
        pfm.measure_fp32_peak(blocks_per_sm=0)
    with pytest.raises(pfm.PfmError):
        pfm.measure_fp32_peak(iters=0)
