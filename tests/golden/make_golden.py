"""Generates the golden fixtures in this directory from the reference's own solvers.

The executables come from oracle/make_ref.sh, which compiles the reference sources
(base-c/base_shll.c, base-c/base_shll_2d.c, base-c/2nd_order_base_shll.c,
base-omp/2nd_order_base_shll.c) with only their problem size / end time changed, float->double
for the FP64 variants and a round-trip output format.  Each fixture stores the reference's final
primitive fields (rho, u, [v,] T per cell, as written by its Save_Results) and its printed step
count.  Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# name -> (executable, columns of results.dat, metadata)
CASES = {
    "ref1d_o1_f32_n64": ("base_shll_f32_n64", [1, 2, 3], dict(dim=1, order=1, nx=64, ny=1, bits=32, t_end=0.2, ic="sod")),
    "ref1d_o1_f64_n64": ("base_shll_f64_n64", [1, 2, 3], dict(dim=1, order=1, nx=64, ny=1, bits=64, t_end=0.2, ic="sod")),
    "ref1d_o1_f32_n256": ("base_shll_f32_n256", [1, 2, 3], dict(dim=1, order=1, nx=256, ny=1, bits=32, t_end=0.2, ic="sod")),
    "ref1d_o1_f64_n256": ("base_shll_f64_n256", [1, 2, 3], dict(dim=1, order=1, nx=256, ny=1, bits=64, t_end=0.2, ic="sod")),
    "ref2d_o1_f32_16x16": ("base_shll_2d_f32_16x16", [2, 3, 4, 5], dict(dim=2, order=1, nx=16, ny=16, bits=32, t_end=0.1, ic="box")),
    "ref2d_o1_f64_32x24": ("base_shll_2d_f64_32x24", [2, 3, 4, 5], dict(dim=2, order=1, nx=32, ny=24, bits=64, t_end=0.1, ic="box")),
    "ref2d_o2_f32_16x16": ("o2_2d_f32_16x16", [2, 3, 4, 5], dict(dim=2, order=2, nx=16, ny=16, bits=32, t_end=0.2, ic="four_shock")),
    "ref2d_o2_f64_32x24": ("o2_2d_f64_32x24", [2, 3, 4, 5], dict(dim=2, order=2, nx=32, ny=24, bits=64, t_end=0.2, ic="four_shock")),
    "refomp_mc_f32_32x32": ("omp_mc_2d_f32_32x32", [2, 3, 4, 5], dict(dim=2, order=2, nx=32, ny=32, bits=32, t_end=0.05, ic="quadrants", limiter=1)),
    "refomp_mc_f64_32x32": ("omp_mc_2d_f64_32x32", [2, 3, 4, 5], dict(dim=2, order=2, nx=32, ny=32, bits=64, t_end=0.05, ic="quadrants", limiter=1)),
}


def main():
    subprocess.run([os.path.join(ROOT, "oracle", "make_ref.sh")], check=True)
    with tempfile.TemporaryDirectory() as wd:
        for name, (exe, cols, meta) in CASES.items():
            steps, prim = O.run_ref(exe, cols, wd)
            np.savez_compressed(os.path.join(OUT, name + ".npz"), prim=prim, steps=steps,
                                **{k: v for k, v in meta.items()})
            print(name, steps, prim.shape)


if __name__ == "__main__":
    main()
