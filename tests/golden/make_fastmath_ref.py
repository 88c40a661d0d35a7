"""Writes fastmath_ref.npz: inputs and correctly rounded exp, log and 1/x
(200-bit mpmath, then rounded to the nearest double) for
tests/test_fastmath_gpu.py.  Run from the repository root:

    python tests/golden/make_fastmath_ref.py
"""
from pathlib import Path

import mpmath as mp
import numpy as np

mp.mp.prec = 200


def main():
    rng = np.random.default_rng(1)
    xe = np.concatenate([rng.uniform(-700, 700, 1500), rng.uniform(0.0, 12.0, 1500),
                         [0.0, -0.0, 1e-300, 0.5 * np.log(2) / 64, 700.0, -700.0]])
    rng = np.random.default_rng(2)
    xl = np.concatenate([10.0 ** rng.uniform(-290, 290, 1500), rng.uniform(50.0, 3000.0, 1500),
                         [1.0, 2.0, 0.5, 1.0 + 2 ** -40, 273.15, 1e-290, 1e290]])
    exp_ref = np.array([float(mp.exp(mp.mpf(float(v)))) for v in xe])
    log_ref = np.array([float(mp.log(mp.mpf(float(v)))) for v in xl])
    rcp_ref = np.array([float(1 / mp.mpf(float(v))) for v in xl])
    out = Path(__file__).with_name("fastmath_ref.npz")
    np.savez_compressed(out, xe=xe, exp=exp_ref, xl=xl, log=log_ref, rcp=rcp_ref)
    print(out)


if __name__ == "__main__":
    main()
