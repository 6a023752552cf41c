"""Generates tests/golden/detector_golden.npz: detections of the reference's
own SingleChannel::MatchedFilter<double> + SingleChannel::Detector<double>
(src/singleChannel/detector.cpp, compiled unchanged into
oracle/_ref/libmflib_ref.so by oracle/build.py) on a seeded single-channel
case, for every detector option combination.  The inputs are stored with
the outputs, so the fixture does not depend on scipy's filters.

Run from the repository root where the reference checkout exists:
    python tests/golden/make_detector_golden.py
"""
import os
import sys

import numpy as np
from scipy.signal import butter, sosfilt
from scipy.signal.windows import hann

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle.orc import Reference  # noqa: E402

FS = 100.0
THR, MIND = 0.5, 100


def case():
    rng = np.random.default_rng(5)

    def bp(x, lo, hi):
        return sosfilt(butter(4, [lo, hi], btype="bandpass", fs=FS, output="sos"), x)

    tps = [bp(rng.standard_normal(300), 2, 8) * hann(300) for _ in range(3)]
    n = 20_000
    x = bp(rng.standard_normal(n), 1, 10)
    for t, tp in enumerate(tps):
        for o in rng.integers(0, n - 300, 4):
            x[o:o + 300] += rng.uniform(0.5, 2) * np.std(x) * tp / np.std(tp) * (1 if t != 1 else -1)
    return tps, x


def main():
    tps, x = case()
    ref = Reference()
    out = {"templates": np.stack(tps), "signal": x, "fs": FS, "threshold": THR, "min_distance": MIND}
    for single in (0, 1):
        for interp in (0, 1, 2):
            for absm in (0, 1):
                r = ref.detect(tps, x, FS, threshold=THR, min_distance=MIND, single=single, interpolation=interp,
                               absolute_maximum=absm, dtype=np.float64)
                for k, v in r.items():
                    out["s%d_i%d_a%d_%s" % (single, interp, absm, k)] = v
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "detector_golden.npz")
    np.savez_compressed(path, **out)
    print(path)


if __name__ == "__main__":
    main()
