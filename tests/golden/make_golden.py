"""Regenerate the golden fixtures of this directory from the reference tree.

Reads the reference's ndarray-serde bincode test fixtures (layout: u8 version,
u64 dims[ndim], u64 len, f64 data[len], C order) and writes them as .npy:

  stress_kernel.npy  <- test/control/stress_kernel.bincode   [3,3,9,9]
                        (src/flowfield/stress_test.rs:82-122)
  ff_test.npy        <- test/flowfield/ff_test.bincode       [3,11,11,11]
                        (src/flowfield/spectral_solver_test.rs:15-65)
  b_test.npy         <- test/magneticfield/b_test.bincode    [3,11,11,11]
                        (src/magnetic_interaction/magnetic_solver_test.rs:43-92)

Usage: python tests/golden/make_golden.py [REFERENCE_ROOT]
"""
import math
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = {
    "stress_kernel.npy": ("test/control/stress_kernel.bincode", 4),
    "ff_test.npy": ("test/flowfield/ff_test.bincode", 4),
    "b_test.npy": ("test/magneticfield/b_test.bincode", 4),
}


def read_ndarray_bincode(path, ndim):
    b = open(path, "rb").read()
    if b[0] != 1:
        raise ValueError(f"{path}: unknown ndarray serde version {b[0]}")
    dims = list(struct.unpack_from("<" + "Q" * ndim, b, 1))
    (n,) = struct.unpack_from("<Q", b, 1 + 8 * ndim)
    if n != math.prod(dims):
        raise ValueError(f"{path}: length {n} does not match dims {dims}")
    off = 1 + 8 * ndim + 8
    return np.frombuffer(b, dtype="<f8", count=n, offset=off).reshape(dims).copy()


def main(ref_root):
    for out, (rel, ndim) in FIXTURES.items():
        a = read_ndarray_bincode(os.path.join(ref_root, rel), ndim)
        np.save(os.path.join(HERE, out), a)
        print(out, a.shape)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <root of the reference checkout>")
    main(sys.argv[1])
