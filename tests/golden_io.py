"""Loading helpers for the golden fixtures in tests/golden/*.npz."""
import glob
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MHD_KEYS = ("prim", "cons", "fbx", "fby", "t", "cycle", "sl_prim", "sl_cons", "sl_fbx", "sl_fby", "sl_t")
HYDRO_KEYS = ("prim", "cons", "t", "cycle", "sl_prim", "sl_cons", "sl_t")


def golden_files(physics):
    return sorted(glob.glob(os.path.join(GOLDEN_DIR, f"{physics}_*.npz")))


def load(path):
    z = np.load(path)
    params = {k[2:]: z[k].item() for k in z.files if k.startswith("p_")}
    inputs = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    outputs = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return params, inputs, outputs


def case_id(path):
    return os.path.basename(path)[:-4]
