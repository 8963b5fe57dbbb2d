"""Host-side pieces of the full-configuration run (CPU only): the
time-to-PSNR reading of a held-out PSNR curve."""
from msplat_gb300.full_run import time_to


def test_time_to_interpolates_the_crossing():
    curve = [(500, 1.0, 20.0), (1000, 2.0, 30.0), (1500, 3.0, 34.0), (2000, 4.0, 35.0)]
    assert time_to(curve, 32.0) == 2.5                  # halfway between 30 and 34 dB
    assert time_to(curve, 35.0) == 4.0                  # reached exactly at the last evaluation
    assert time_to(curve, 19.0) == 1.0                  # already there at the first one
    assert time_to(curve, 35.5) is None                 # never reached
    assert time_to([], 10.0) is None


def test_time_to_takes_the_first_crossing():
    curve = [(500, 1.0, 20.0), (1000, 2.0, 31.0), (1500, 3.0, 29.0), (2000, 4.0, 33.0)]
    assert abs(time_to(curve, 30.0) - (1.0 + 10.0 / 11.0)) < 1e-12
