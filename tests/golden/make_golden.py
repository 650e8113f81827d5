"""Generate the golden fixtures from the reference toolkit's own C-OMP code.

Runs every case of ``cases.py`` through ``oracle/_ref/libcilreg_ref.so`` (the
reference sources compiled by ``make -C oracle ref``) and stores inputs (and
the FGP-dTV reference images), outputs, infovectors and TV energies in
``reference_outputs.npz``; also the FGP and TGV cases on a second 3D input
whose x extent is a multiple of 4 (``staged_cases``).  The reference's
non-linear diffusion updates in place, so it is run with one OpenMP thread
(lexicographic order), the only deterministic setting.

Usage (where the reference sources exist):
    python tests/golden/make_golden.py
"""
import os
import sys

os.environ["OMP_NUM_THREADS"] = "1"  # deterministic order for the in-place diffusion sweep

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "ccpi-regularisation-toolkit_gb300"))
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

import cases as C  # noqa: E402
import oracle as O  # noqa: E402


def main():
    O.build(ref=True)
    if O.ref_lib() is None:
        raise SystemExit("the reference C-OMP library could not be built (are its sources present?)")
    arrays = {}
    for dim in (2, 3):
        arrays[f"input_{dim}d"] = C.make_input(dim)
        arrays[f"ref_{dim}d"] = C.make_ref(dim)
        for lam, typ in C.ENERGY:
            e = O.tv_energy(arrays[f"input_{dim}d"], arrays[f"ref_{dim}d"], lam, typ, use_ref=True)
            arrays[f"energy_{dim}d_{lam}_{typ}"] = np.float32(e)
            print(f"energy {dim}d lambda={lam} type={typ}: {e!r}")
    for case in C.cases():
        x = arrays[f"input_{case['dim']}d"]
        out, info = C.run_oracle(case, x, use_ref=True, ref=arrays[f"ref_{case['dim']}d"])
        arrays[f"out_{case['key']}"] = out
        arrays[f"info_{case['key']}"] = info
        print(f"{case['key']:24s} iters={int(info[0]):4d} re={info[1]:.3e}")
    arrays["input_3dx4"] = C.make_input_x4()
    for case in C.staged_cases():
        out, info = C.run_oracle(case, arrays["input_3dx4"], use_ref=True)
        arrays[f"out_{case['key']}"] = out
        arrays[f"info_{case['key']}"] = info
        print(f"{case['key']:24s} iters={int(info[0]):4d} re={info[1]:.3e}")
    path = os.path.join(HERE, "reference_outputs.npz")
    np.savez_compressed(path, **arrays)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
