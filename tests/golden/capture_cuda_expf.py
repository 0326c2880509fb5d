"""Record CUDA's float32 expf of the Ising fixture's acceptance arguments.

    python tests/golden/capture_cuda_expf.py      (needs a GPU and libmcgb)

The reference accepts an Ising flip when u < expf(-beta * dE) evaluated by
CUDA's float32 expf, which is not correctly rounded everywhere (2 ulp bound).
The Ising sweep fixture therefore takes those five values per temperature as
an input: this script writes them, as float32 bit patterns, to
``ising_cuda_expf.json``; make_golden.py reads the file and the golden tests
check it against the exact exponential (CPU) and against expf on the GPU.
"""

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
sys.path.insert(0, str(HERE.parents[1] / "gpu-monte-carlo_gb300"))

ISING_TEMPERATURES = (1.5, 2.269, 3.0)


def exponent_arguments(betas):
    """float32 arguments -beta * dE for dE = -8, -4, 0, 4, 8 (J = 1), shape (R, 5)."""
    k = np.array([-8, -4, 0, 4, 8], np.float32)
    return (-np.asarray(betas, np.float32)[:, None] * k[None, :]).astype(np.float32)


def main():
    from mcgb import _lib, device
    betas = (1 / np.array(ISING_TEMPERATURES)).astype(np.float32)
    args = exponent_arguments(betas)
    x, y = device.to_device(args), device.device_array(args.shape, np.float32)
    _lib.call("mcgb_expf", x.cptr, y.cptr, args.size, _lib.stream_handle())
    table = y.copy_to_host()
    out = {"temperatures": list(ISING_TEMPERATURES),
           "arguments_f32_bits": [[f"{int(v):08x}" for v in row] for row in args.view(np.uint32)],
           "expf_f32_bits": [[f"{int(v):08x}" for v in row] for row in table.view(np.uint32)]}
    (HERE / "ising_cuda_expf.json").write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out))


if __name__ == "__main__":
    main()
