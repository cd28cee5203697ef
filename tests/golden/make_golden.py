"""Generate the golden fixtures under tests/golden/ from the reference itself.

Runs the reference's own headers (built by `make -C oracle ref` against the
Eigen-subset shim, from the reference sources) on small seeded cases and
stores points, tree lists, NCA pivots, storage counts, matvec outputs, the
dense product and GMRES results. Needs the reference tree; the committed
.npz files are what the tests read (no test reads the reference).

    python tests/golden/make_golden.py <reference checkout> [case ...]
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)
from h2wdump import read_dump, write_input  # noqa: E402
from h2weak_gb300 import synth  # noqa: E402

# name: dim, form, n_param, nLevels, leaf_param, tol_pow, choice, points (None = grid), gmres tol_pow
CASES = {
    "g1d_n_rbf": (1, "n", 2048, 5, 64, 10, 1, None, 10),
    "g1d_sn_ie": (1, "sn", 2048, 5, 64, 10, 0, None, 10),
    "g2d_n_ie": (2, "n", 48, 3, 6, 10, 0, None, 10),
    "g2d_sn_rbf": (2, "sn", 48, 3, 6, 10, 1, None, 10),
    "g3d_n_rbf": (3, "n", 16, 2, 4, 8, 1, None, 10),
    "g3d_sn_ie": (3, "sn", 16, 2, 4, 8, 0, None, 10),
    "g2d_n_rand": (2, "n", 0, 3, 0, 8, 1, ("uniform", 2, 3000), 10),
    "g3d_n_rand": (3, "n", 0, 2, 0, 8, 1, ("uniform", 3, 4000), 10),
    # non-nested H* (USE_HODLRdD)
    "g2d_nn_rbf": (2, "nn", 48, 3, 6, 10, 1, None, 10),
    "g3d_nn_ie": (3, "nn", 16, 2, 4, 8, 0, None, 10),
    "g2d_nn_rand": (2, "nn", 0, 3, 0, 8, 0, ("uniform", 2, 3000), 10),
    # complex Helmholtz kernel (USE_Helm, choice 2): complex vectors
    "g3d_n_helm": (3, "n_helm", 16, 2, 4, 10, 2, None, 10),
    "g3d_sn_helm": (3, "sn_helm", 16, 2, 4, 8, 2, None, 10),
    "g3d_n_helm_rand": (3, "n_helm", 0, 2, 0, 8, 2, ("uniform", 3, 4000), 10),
    # complex 2D Hankel kernel (USE_Hankel, choice 10), the reference built against the
    # Boost Bessel stand-in (oracle/boost_shim): complex vectors
    "g2d_n_hankel": (2, "n_hankel", 48, 3, 6, 10, 10, None, 10),
    "g2d_sn_hankel": (2, "sn_hankel", 48, 3, 6, 8, 10, None, 10),
    "g2d_n_hankel_rand": (2, "n_hankel", 0, 3, 0, 8, 10, ("uniform", 2, 3000), 10),
    # the complex kernels in the non-nested H* form (USE_HODLRdD with USE_Helm / USE_Hankel)
    "g3d_nn_helm": (3, "nn_helm", 16, 2, 4, 8, 2, None, 10),
    "g2d_nn_hankel": (2, "nn_hankel", 48, 3, 6, 8, 10, None, 10),
    # ties of the partition rule: random points with about 30 % of their coordinates moved
    # down onto the grid of quarters, so that many lie exactly on the split planes of
    # levels 1-3 (and on the domain's lower faces); duplicates removed
    "g2d_n_snap": (2, "n", 0, 3, 0, 8, 1, ("snapped", 2, 3000), 10),
    "g2d_sn_snap": (2, "sn", 0, 3, 0, 8, 1, ("snapped", 2, 3000), 10),
    "g3d_n_snap": (3, "n", 0, 3, 0, 8, 1, ("snapped", 3, 4000), 10),
}
FORMS = {"n": 0, "sn": 1, "nn": 2, "n_helm": 0, "sn_helm": 1, "nn_helm": 2, "n_hankel": 0, "sn_hankel": 1,
         "nn_hankel": 2}
LISTS = ["charge", "nbr", "il", "isvertex", "far_check", "far_charge", "ver_check", "ver_charge", "sn_row", "sn_col"]


def run_case(name, spec):
    dim, form, npar, nlev, leaf, tol, ch, pts, gtol = spec
    if pts is not None:
        kind, n = pts[0], pts[2]
        pts = synth.uniform_points(synth.config_seed(40 + dim, 0), n, dim)
        if kind == "snapped":
            snap = synth.uniform01(synth.config_seed(44, dim), n * dim).reshape(n, dim) < 0.3
            pts = np.where(snap, np.floor(pts * 4.0) / 4.0, pts)
            _, first = np.unique(pts, axis=0, return_index=True)
            pts = np.ascontiguousarray(pts[np.sort(first)])
        N = len(pts)
    else:
        N = npar ** dim
    cplx = form.endswith(("_helm", "_hankel"))
    if cplx:  # real and imaginary parts from separate streams
        vecs = [synth.normal(synth.config_seed(90, v), N) + 1j * synth.normal(synth.config_seed(92, v), N)
                for v in range(2)]
        xtrue = synth.normal(synth.config_seed(91, 0), N) + 1j * synth.normal(synth.config_seed(93, 0), N)
    else:
        vecs = [synth.normal(synth.config_seed(90, v), N) for v in range(2)]
        xtrue = synth.normal(synth.config_seed(91, 0), N)
    inp, out = "/tmp/golden_in_%s.bin" % name, "/tmp/golden_out_%s.bin" % name
    write_input(inp, pts, vecs, xtrue, dense=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "ref%dd_%s" % (dim, form))
    r = subprocess.run([exe, str(npar), str(nlev), str(leaf), "1", str(tol), str(ch), inp, out, "500", str(gtol)],
                       capture_output=True, text=True, check=True)
    d = read_dump(out)
    vec = (lambda a: a.view(np.complex128)) if cplx else (lambda a: a)
    rec = {"spec": np.array([dim, FORMS[form], npar, nlev, leaf, tol, ch, gtol, N], dtype=np.int64),
           "points": d["points"].reshape(N, dim), "vecs": np.stack(vecs), "xtrue": xtrue,
           "memory": d["memory"], "matvec": vec(d["matvec"]).reshape(2, N), "dense_matvec": vec(d["dense_matvec"]),
           "gmres_rhs": vec(d["gmres_rhs"]), "gmres_x": vec(d["gmres_x"]), "gmres_stats": d["gmres_stats"]}
    for nm in LISTS:
        rec[nm + "_ptr"] = d[nm + ".ptr"]
        rec[nm + "_val"] = d[nm + ".val"]
    if "uv_rank" in d:
        rec["uv_rank"] = d["uv_rank"]
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
    return r.stdout.strip().splitlines()[-1]


if __name__ == "__main__":
    # python tests/golden/make_golden.py <reference checkout> [case ...]
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "REF=" + sys.argv[1]], check=True)
    names = sys.argv[2:] or list(CASES)
    for name in names:
        print(name, run_case(name, CASES[name]))
