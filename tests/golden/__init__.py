"""Golden fixtures produced by the reference's own sources (make_golden.py)."""
import dataclasses
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = ("heated16_2steps", "cooled24_gravity_switch", "shipped24_1step")
STATS_NAMES = ("stats16_3steps",)
SCALAR_NAMES = ("scalar16_source_2steps", "scalar24_meangrad_2steps")


def load(name):
    """Returns (Params, State, dict of reference outputs, nsteps, as_shipped)."""
    from tpm import inputs
    from tpm.params import Params

    z = np.load(os.path.join(HERE, name + ".npz"))
    p = Params(**json.loads(str(z["params"])))
    part = {q: z[f"in_part_{q}"] for q in list(inputs.PQ) + ["flag"]}
    s = inputs.State(RU=z["in_RU"], Rho=z["in_Rho"], P=z["in_P"], part=part,
                     P0=float(z["in_P0"]), PS=z["in_PS"] if "in_PS" in z.files else None)
    ref = {k: z[k] for k in ("RU", "RU_int", "Rho", "P", "C", "Q")}
    ref["part"] = {q: z[f"part_{q}"] for q in list(inputs.PQ) + ["flag", "RHS_T"]}
    ref["P0"] = float(z["P0"])
    ref["T_cur"] = float(z["T_cur"])
    ref["stats"] = {k[5:]: z[k] for k in z.files if k.startswith("stat_")}
    if "PS" in z.files:
        ref["PS"] = z["PS"]
    return p, s, ref, int(z["nsteps"]), bool(int(z["as_shipped"]))
