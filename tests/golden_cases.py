"""Loading of the golden fixtures made by tests/golden/make_golden.py."""

import json
import os

import numpy as np

from oracle import seemps_oracle as so

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys_path_inserted = False


def load_case(name: str):
    """Return (params, mps, mpo, golden-dict); regenerates the seeded inputs."""
    import importlib.util

    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    meta = json.loads(bytes(z["meta"]).decode())
    p = meta["params"]
    mps, mpo = mg.make_inputs(p)
    same_inputs = mg.input_hash(mps, mpo) == meta["input_sha256"]
    g = {k: z[k] for k in z.files if k != "meta"}
    if "split_full_len" not in g:
        g["split_full_len"] = g["split_len"]
    offs = np.concatenate([[0], np.cumsum(g["split_len"])])
    g["splits_s"] = [g["split_s"][offs[i]:offs[i + 1]] for i in range(len(g["split_len"]))]
    return p, mps, mpo, g, same_inputs


def strategy_for(p, module=so):
    st = module.DEFAULT_STRATEGY.replace(
        tolerance=p["tol"], max_bond_dimension=p["maxchi"], max_sweeps=p["sweeps"])
    if p.get("stol") is not None:
        st = st.replace(simplification_tolerance=p["stol"])
    return st


def run_oracle(p, mps, mpo, rec=None):
    st = strategy_for(p)
    if p["kind"] in ("mpo_apply", "laplacian"):
        return so.mpo_apply(mpo, mps, st, rec=rec), so.mpo_apply(mpo, mps, st, simplify_flag=False).tensors
    if p["kind"] == "euler":
        Lx = [so.mpo_multiply_tensor(O, B) for O, B in zip(mpo, mps)]
        return so.simplify_mps_sum([1.0, p["dt"]], [mps, Lx], st, rec=rec), None
    return so.simplify(mps, st, rec=rec), mps


def truncation_cases():
    with open(os.path.join(GOLDEN, "truncation_cases.json")) as f:
        d = json.load(f)
    return [(np.array(d["vectors"][c["v"]]), c) for c in d["cases"]]


CASE_NAMES = ["c1_small", "c1", "lap_small", "lap_n30_chi32", "euler_small", "simplify_real",
              "c2", "northstar"]
