"""Shared helpers of the test suite: fixture loading and bit-exact comparison
of CA results (the oracle's result/contact layouts and the library's share
their leading fields)."""
from __future__ import annotations

import os

import numpy as np

from c2a_gb300 import meshes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# result fields compared bit for bit between implementations
RESULT_FIELDS = ["collisionfree", "numCA", "translation", "num_contact", "toc", "distance", "mint", "num_bv_tests",
                 "num_tri_tests", "seed_a", "seed_b"]
CONTACT_FIELDS = ["type_a", "type_b", "fid_a", "fid_b", "tri_a", "tri_b", "pa", "pb", "distance"]


def bits(x) -> bytes:
    a = np.asarray(x)
    if a.dtype.kind == "f":
        a = a.astype(np.float64)
    return np.ascontiguousarray(a).tobytes()


def load_fixture(name: str):
    """(meshes, qint, poses, params, expected results, contacts, contact offsets)."""
    z = np.load(os.path.join(GOLDEN, f"{name}_ref.npz"))
    ms = [meshes.Mesh(f"{name}{i}", z[f"mesh{i}_verts"], z[f"mesh{i}_faces"], np.zeros((1, 3)), 0.0)
          for i in range(int(z["num_meshes"]))]
    p = z["params"]
    params = dict(tol_d=float(p[0]), tol_t=float(p[1]), toc_delta=float(p[2]), contact_abs=float(p[3]),
                  with_contacts=int(p[4]), max_iters=int(p[5]), qsize=40)
    return ms, z["qint"], z["poses"], params, z["results"], z["contacts"], z["contact_offsets"]


def result_mismatches(got, exp, got_contacts=None, exp_contacts=None, exp_offsets=None, fields=RESULT_FIELDS):
    """Indices of queries whose results (and contacts, when given) differ in any bit.

    got_contacts: (n, slots) per-query contact rows in visiting order;
    exp_contacts/exp_offsets: the flattened expected contacts."""
    bad = []
    for q in range(len(exp)):
        ok = all(bits(got[q][f]) == bits(exp[q][f]) for f in fields)
        if ok and not exp[q]["collisionfree"]:
            ok = bits(got[q]["R_toc"]) == bits(exp[q]["R_toc"]) and bits(got[q]["T_toc"]) == bits(exp[q]["T_toc"])
            if ok and got_contacts is not None:
                n = int(exp[q]["num_contact"])
                g = got_contacts[q][:n]
                e = exp_contacts[exp_offsets[q]:exp_offsets[q + 1]]
                ok = len(g) == len(e) and all(bits(g[f]) == bits(e[f]) for f in CONTACT_FIELDS)
        if not ok:
            bad.append(q)
    return bad


def describe(got, exp, q, fields=RESULT_FIELDS) -> str:
    return "query %d:\n  got %s\n  exp %s" % (q, {f: got[q][f] for f in fields}, {f: exp[q][f] for f in fields})
