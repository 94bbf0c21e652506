"""Generate the golden vectors under tests/golden/ from the Modal-CMB
reference's own sources, compiled in place (oracle/_ref, `make -C oracle ref`).

Run in a container that has the reference checkout:
    python tests/golden/make_golden.py
The fixtures are small .npz files; tests read them without the reference.
Inputs are rebuilt by the tests from modal_gb300's synthetic-workload
builders with the same arguments, and their checksums are stored alongside.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "modal-cmb_gb300"))
import modal_gb300 as M  # noqa: E402
import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, OUT)


def inputs_digest(q, tr, cl):
    return np.array([q.sum(), (q * q).sum(), tr.sum(), cl.sum()])


def dense_input(size):
    """Seeded-free smooth test bispectrum for the serial dense form (also rebuilt by the tests)."""
    l = np.arange(size, dtype=np.float64)
    l[0] = 1.0
    raw = np.einsum("i,j,k->ijk", l ** -1.2, l ** -0.7, l ** -1.5)
    return (raw + raw.transpose(1, 2, 0) + raw.transpose(2, 0, 1)) / 3.0


def transfer_inputs(lmax, Pp, xsize):
    """Synthetic radial grid and transfer functions q~_p(l, x) (also rebuilt by the tests)."""
    xvec = np.linspace(1000.0, 12000.0, xsize)
    l = np.arange(lmax + 1.0)
    qt = np.zeros((xsize, Pp, lmax + 1))
    for xi, x in enumerate(xvec):
        for p in range(Pp):
            qt[xi, p] = np.cos((p + 1) * x / 4000.0) * np.sin(0.1 * l * (1 + p) + x / 3000.0) / (1.0 + l)
    return xvec, qt


def main():
    ref = O.Ref()
    # 1. asy() Gauss-Legendre nodes/weights
    gl = {}
    for n in (31, 91, 751, 1501, 3001):
        x, w = ref.asy(n)
        gl[f"x{n}"], gl[f"w{n}"] = x, w
    np.savez_compressed(os.path.join(OUT, "gl_asy.npz"), **gl)

    # 2. basis_functions_legendre for config 1's basis (l = 2..500, pmax = 9)
    vals = np.arange(2, 501, dtype=np.float64)
    np.savez_compressed(os.path.join(OUT, "basis_legendre.npz"), values=vals,
                        basis=ref.basis_legendre(vals, 9, 2.0, 500.0))

    # 3. calculate_geometric at seeded tetrapyd points and off-tetrapyd points
    rng = np.random.default_rng(7)
    pts = rng.integers(0, 2500, size=(2000, 3)).astype(np.int32)
    geo = np.array([ref.L.ref_geometric(int(a), int(b), int(c)) for a, b, c in pts])
    np.savez_compressed(os.path.join(OUT, "geometric.npz"), pts=pts, geo=geo)

    # 4. tetrapyd walk / decomposition
    walk, n = ref.tetrapyd_walk(2, 30, 400)
    counts = {f"{a}_{b}": ref.tetrapyd_walk(a, b, 0)[1] for a, b in [(2, 3), (2, 10), (3, 31), (2, 100), (5, 64)]}
    dec = ref.decompose(8, 2, 100)
    np.savez_compressed(os.path.join(OUT, "tetrapyd.npz"), walk=walk[:400], walk_count=n, decompose=dec,
                        **{"count_" + k: v for k, v in counts.items()})

    # 5. serial dense form: modify_bispectrum + calculate_modes at size 41 (l = index),
    #    basis for l = 2..40, P = 4; input: a seeded smooth bispectrum
    lmax, P, size = 40, 4, 41
    q, tr, cl = M.workload(lmax, P)
    ref.setup(2, lmax, q, tr, cl)
    raw = dense_input(size)
    vec = np.arange(size, dtype=np.int32)
    mod = ref.modify_bispectrum(raw, vec)
    beta = ref.calculate_modes(mod)
    np.savez_compressed(os.path.join(OUT, "modes_dense.npz"), modified=mod, beta=beta, lmax=lmax, P=P)

    # 6. late x primordial transfer Gamma (calculate_gamma_2d over all (m, n))
    out = {}
    for name, lmax, P, Pp, xsize in [("a", 40, 3, 3, 30), ("b", 90, 4, 5, 41)]:
        q, tr, cl = M.workload(lmax, P)
        ref.setup(2, lmax, q, tr, cl)
        xvec, qt = transfer_inputs(lmax, Pp, xsize)
        prim = M.mode_triples(Pp)
        out["gamma_" + name] = ref.gamma_transfer(xvec, qt, prim, 0.7)
        out["dims_" + name] = np.array([lmax, P, Pp, xsize])
    np.savez_compressed(os.path.join(OUT, "gamma_transfer.npz"), **out)

    # 7. Gamma (calculate_orthol over all pairs) and projection beta
    #    small: lmax=60, P=4; config 1: lmax=500, P=10 (220 modes)
    for name, lmax, P, S in [("small", 60, 4, 4), ("cfg1", 500, 10, 4)]:
        q, tr, cl = M.workload(lmax, P)
        ref.setup(2, lmax, q, tr, cl)
        with O.quiet_stdout():
            ref.init_gamma()
        G, _ = ref.gamma(nranks=8)
        shapes = M.separable_shapes(lmax, S // 2, seed=0) + M.bump_shapes(S - S // 2, seed=1)
        beta = np.stack([ref.project(s, nthreads=8) for s in shapes])
        np.savez_compressed(os.path.join(OUT, f"gamma_{name}.npz"), gamma=G, beta=beta, lmax=lmax, P=P, S=S,
                            digest=inputs_digest(q, tr, cl))
        print(name, "done", G.shape, beta.shape)


def prune_golden():
    """8. greedy basis pruning: the reference's basis_optimisation_mpi.c main()
    (oracle/_ref/basis_prune_ref) on a Gamma of 35 modes with two failed modes,
    and on a seeded 60 x 60 SPD matrix."""
    q, tr, cl = M.workload(120, 5)
    orc = O.Oracle()
    mu, w = orc.gl_nodes(181)
    G = orc.gamma(orc.mij(orc.legendre_table(mu, 120), 2, 120, q), w, tr)
    fail = np.array([3, 7])
    order_a, lam_a = O.ref_basis_prune(G, fail)
    X = np.random.default_rng(0).standard_normal((60, 80))
    R = X @ X.T
    order_b, lam_b = O.ref_basis_prune(R)
    np.savez_compressed(os.path.join(OUT, "basis_prune.npz"), gamma_a=G, fail_a=fail, order_a=order_a, lam_a=lam_a,
                        gamma_b=R, order_b=order_b, lam_b=lam_b)
    print("basis_prune done", order_a.size, order_b.size)


def pol_inputs(lmaxT=50, lmaxE=60, lminE=3, PT=4, PE=4):
    """Polarised case: T basis on 2..lmaxT, E basis on lminE..lmaxE with its own
    weight, TTE/TEE/EEE triples in the find_perm_late_XXX conventions."""
    cl = M.synthetic_cl(max(lmaxT, lmaxE))
    qT = M.weighted_q(M.legendre_q(2, lmaxT, PT), cl, 2)
    qE = M.weighted_q(M.legendre_q(lminE, lmaxE, PE), cl * 2.0, lminE)
    ttt = M.mode_triples(PT)
    N = len(ttt)
    tte = np.array([(p, r, s) for p in range(PT) for r in range(p, PT) for s in range(PE)][:N], dtype=np.int32)
    tee = np.array([(t, a, b) for t in range(PT) for a in range(PE) for b in range(a, PE)][:N], dtype=np.int32)
    eee = M.mode_triples(PE)[:N]
    return cl, qT, qE, ttt, tte, tee, eee


def pol_transfer_inputs(lmax=40, lmaxE=34, lminE=2, P=3, PE=3, Pp=3, xsize=30):
    """Polarised transfer case: T and E bases, TTE/TEE/EEE late triples, synthetic
    TT/TE/EE spectra with beams, noise and sky fractions, T and E transfer
    functions on one radial grid.  lmaxE <= lmax."""
    l = np.arange(lmax + 1.0)
    ls = np.maximum(l, 2.0)
    cl_tt = 1e3 / (ls * (ls + 1)) * np.exp(-(l / 1500.0) ** 2)
    cl_ee = 0.05 * cl_tt
    cl_te = 0.3 * np.sqrt(cl_tt * cl_ee) * np.cos(l / 7.0)
    b_tt = np.exp(-l * (l + 1) * 1e-5)
    b_ee = np.exp(-l * (l + 1) * 2e-5)
    b_te = np.sqrt(b_tt * b_ee)
    n_tt, n_ee, n_te = 1e-4 * np.ones_like(l), 3e-4 * np.ones_like(l), 1e-6 * np.ones_like(l)
    spec9 = np.stack([cl_tt, cl_te, cl_ee, b_tt, b_te, b_ee, n_tt, n_te, n_ee])
    cl_total = (b_tt ** 2 * cl_tt + n_tt) / b_tt ** 2  # the TT weight's C_l + N_l/b_l^2
    qT = M.legendre_q(2, lmax, P)
    qE = M.legendre_q(lminE, lmaxE, PE) * 0.7
    ttt = M.mode_triples(P)
    N = len(ttt)
    tte = np.array([(p, r, s) for p in range(P) for r in range(p, P) for s in range(PE)][:N], dtype=np.int32)
    tee = np.array([(t, a, b) for t in range(P) for a in range(PE) for b in range(a, PE)][:N], dtype=np.int32)
    eee = M.mode_triples(PE)[:N]
    xvec, qtT = transfer_inputs(lmax, Pp, xsize)
    _, qtE = transfer_inputs(lmax, Pp, xsize)
    qtE = qtE * 0.5 + 0.1 * np.roll(qtT, 1, axis=1)
    prim = M.mode_triples(Pp)
    return dict(lmax=lmax, lmaxE=lmaxE, lminE=lminE, spec9=spec9, cl_total=cl_total, qT=qT, qE=qE, ttt=ttt, tte=tte,
                tee=tee, eee=eee, xvec=xvec, qtT=qtT, qtE=qtE, prim=prim, fsky_t=0.7, fsky_e=0.5, dphi=0.7)


def pol_transfer_golden():
    """10. polarised transfer Gamma: calculate_gamma_2d's four results."""
    d = pol_transfer_inputs()
    ref = O.Ref()
    ref.setup(2, d["lmax"], d["qT"], d["ttt"], d["cl_total"])
    ref.setup_pol(d["lminE"], d["lmaxE"], d["qE"], d["tte"], d["tee"], d["eee"])
    G = ref.gamma_transfer_pol(d["spec9"], d["fsky_t"], d["fsky_e"], d["xvec"], d["qtT"], d["qtE"], d["prim"], d["dphi"])
    nmu = 3 * d["lmax"] // 2 + 1
    x, w = ref.asy(nmu)
    np.savez_compressed(os.path.join(OUT, "gamma_transfer_pol.npz"), gamma=G, nodes=x, weights=w)
    print("gamma_transfer_pol done", G.shape)


def prim_inputs(kmax_i=40, Pp=4):
    """Primordial k-grid case: cosine basis on grid indices 0..kmax_i, all
    p <= r <= s < Pp triples, two shapes (one separable, one bump)."""
    x = np.arange(kmax_i + 1) / kmax_i
    basis = np.stack([np.cos(np.pi * p * x) + 0.1 * p * x for p in range(Pp)], axis=1)
    prim = M.mode_triples(Pp)
    shapes = M.separable_shapes(kmax_i, 1, 3, 1, 2) + M.bump_shapes(1, 4)
    for sh in shapes:  # tables on grid indices 1..kmax_i (index 0 unused with kmin = 1)
        if sh["kind"] == 0:
            sh["tab"][:, :, 0] = 0.0
    return basis, prim, shapes


def prim_golden():
    """11. primordial k-space side: calculate_ortho, calculate_eigen and
    integrate_template2 on the grid tetrapyd (reference in place)."""
    ref = O.Ref()
    out = {}
    for name, kmin, kmax_i, kmax in [("a", 1, 40, 0.2), ("b", 3, 57, 1.5)]:
        basis, prim, shapes = prim_inputs(kmax_i)
        out["ortho_" + name] = ref.prim_ortho(kmin, kmax_i, kmax, basis, prim)
        for n, sh in enumerate(shapes):
            a, n2 = ref.prim_eigen(kmin, kmax_i, kmax, basis, prim, sh)
            out[f"alpha_{name}{n}"] = a
            out[f"norm2_{name}{n}"] = np.array([n2])
        out["grid_" + name] = np.array([kmin, kmax_i, kmax])
    np.savez_compressed(os.path.join(OUT, "prim.npz"), **out)
    print("prim done")


def pol_golden():
    """9. polarised Gamma: calculate_orthol's four results with do_polarisation."""
    lmaxT, lmaxE, lminE = 50, 60, 3
    cl, qT, qE, ttt, tte, tee, eee = pol_inputs(lmaxT, lmaxE, lminE)
    ref = O.Ref()
    ref.setup(2, lmaxT, qT, ttt, cl)
    ref.setup_pol(lminE, lmaxE, qE, tte, tee, eee)
    with O.quiet_stdout():
        ref.init_gamma()
    G = ref.gamma_pol()
    nmu = 3 * max(lmaxT, lmaxE) // 2 + 1
    x, w = ref.asy(nmu)
    np.savez_compressed(os.path.join(OUT, "gamma_pol.npz"), gamma=G, nodes=x, weights=w,
                        dims=np.array([lmaxT, lmaxE, lminE]))
    print("gamma_pol done", G.shape)


def gamma_3d_golden():
    """12. 3D transfer Gamma: calculate_gamma_TTT_3D_nested through gamma_3d_host's
    set-up (reference in place), late and primordial term counts equal."""
    ref = O.Ref()
    out = {}
    for name, (lmax, P, Pp, xsize, dphi) in {"a": (40, 3, 3, 30, 0.7), "b": (63, 4, 4, 37, 1.3)}.items():
        q, tr, cl = M.workload(lmax, P)
        xvec, qt = transfer_inputs(lmax, Pp, xsize)
        ref.setup(2, lmax, q, tr, cl)
        out["gamma_" + name] = ref.gamma_3d(xvec, qt, M.mode_triples(Pp), dphi)
        out["dims_" + name] = np.array([lmax, P, Pp, xsize])
        out["dphi_" + name] = np.array([dphi])
    np.savez_compressed(os.path.join(OUT, "gamma_3d.npz"), **out)
    print("gamma_3d done")


def files_golden():
    """14. The reference's data-store code on the synthetic inputs of
    tests/golden/files_inputs.py, one INI case per order_late (1-10): file
    names (initilise), mode lists (set_terms_prim, set_terms_late), spectra
    (load_cl, load_BN, load_lens, load_TL), basis tables (create_basis_late)
    and the transfer files read back (read_qtilde; written by
    modal_files.write_qtilde).  Directory prefixes are stored as {DIR}/."""
    import json
    import shutil

    import modal_files as mf
    from files_inputs import CASES, qtilde_tables, write_case
    ref = O.RefFiles()
    out = {}
    for name, cs in CASES.items():
        ol, op, pol, lens, tmin, tmax, emin, emax, terms, absolute = cs
        d = f"/tmp/mfg_{name}/"
        shutil.rmtree(d, ignore_errors=True)
        os.makedirs(d)
        ini = write_case(d, name)
        ref.load(ini)
        out[f"{name}_names"] = np.array(json.dumps({k: v.replace(d, "{DIR}/") for k, v in ref.names().items()}))
        t = ref.terms(terms, pol)
        for k in ("prim", "ttt", "tte", "tee", "eee"):
            if k in t:
                out[f"{name}_{k}"] = t[k]
        out[f"{name}_pmax"] = np.array([t["pmax_prim"], t["pmax_T"], t["pmax_E"]])
        x, qt, qe = qtilde_tables(name, t["pmax_prim"] + 1)
        mf.write_qtilde(mf.read_ini(ini), x, qt, qe if pol else None)
        out[f"{name}_spectra"] = ref.spectra(tmax, True, True)
        bt, be = ref.basis(tmax - tmin + 1, t["pmax_T"] + 1, (emax - emin + 1) if pol else 0, t["pmax_E"] + 1)
        out[f"{name}_basis_T"] = bt
        if pol:
            out[f"{name}_basis_E"] = be
        q = ref.qtilde(t["pmax_prim"] + 1, pol)
        for k, v in q.items():
            out[f"{name}_q_{k}"] = v
        shutil.rmtree(d, ignore_errors=True)
    np.savez_compressed(os.path.join(OUT, "files_ref.npz"), **out)
    print("files_ref done")


def basis_families_golden():
    """13. basis_functions.c's families (legendre, fourier, sinlog, bi) on
    l = 2..700 and on a grid that starts at 0 (sinlog's small-value branch)."""
    ref = O.Ref()
    out = {}
    for name, (lo, hi, pmax) in {"a": (2, 700, 30), "b": (0, 120, 9)}.items():
        v = np.arange(lo, hi + 1, dtype=np.float64)
        vmin = max(lo, 1e-3) if name == "b" else lo  # sinlog takes log(v/min)
        for kind, fam in enumerate(("legendre", "fourier", "sinlog", "bi")):
            out[f"{fam}_{name}"] = ref.basis_family(kind, v, pmax, vmin, hi)
        out["dims_" + name] = np.array([lo, hi, pmax, vmin])
    np.savez_compressed(os.path.join(OUT, "basis_families.npz"), **out)
    print("basis_families done")


if __name__ == "__main__":
    if sys.argv[1:] == ["prune"]:
        prune_golden()
    elif sys.argv[1:] == ["pol"]:
        pol_golden()
        pol_transfer_golden()
    elif sys.argv[1:] == ["prim"]:
        prim_golden()
    elif sys.argv[1:] == ["g3d"]:
        gamma_3d_golden()
    elif sys.argv[1:] == ["basis"]:
        basis_families_golden()
    elif sys.argv[1:] == ["files"]:
        files_golden()
    else:
        main()
        prune_golden()
        pol_golden()
        pol_transfer_golden()
        prim_golden()
        gamma_3d_golden()
        basis_families_golden()
        files_golden()
