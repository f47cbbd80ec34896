"""Extract golden vectors from the Elfel.jl test suite into JSON fixtures.

The reference (Elfel.jl v0.4.0) is Julia and cannot run in this image, so its
known-answer tests are read as text and their literal values are written to
``tests/golden/*.json``.  Only numbers that the reference's own tests assert
are extracted; nothing is computed here.

Run from the repository root with ``ELFEL_REFERENCE`` set to a checkout of
the reference project (required; there is no default):

    ELFEL_REFERENCE=/path/to/Elfel.jl python tests/golden/make_golden.py

Sources (file:line in the reference project):
  test/test_assemblers.jl:6-34      7x7 COO assembly with duplicate summation
  test/test_feiterators.jl:21-71    qmesh connectivity and scalar DOF numbers
  test/test_feiterators.jl:140-172  3-component DOF numbers
  test/test_feiterators.jl:88-119   element-by-element matrix A
  test/test_heat.jl:110             T3 N=4 solution vector
  test/test_stokes.jl:130           Taylor-Hood DOF counts at N=100
  test/test_stokes.jl:551-558       Taylor-Hood error norms N=4,8,16
  test/test_stokes.jl:777-780       vector-Laplacian Taylor-Hood error norms N=4
  test/test_qpiterators.jl:22-61    basis values, gradients and weights
  test/test_refshapes.jl:26-29      3-point triangle rule
  test/test_fefields.jl:13-52       numbering counts on mt3gen3
  test/test_refshapes.jl:1-146      interval, square, triangle, tetrahedron rules
  test/test_felements.jl:1-158      L2, T4, FEL2_Q4, FEL2_T4, FEL2_T3 elements
  test/test_fespaces.jl:85-172      T3 with a bubble: features, DOF layout
  test/test_heat.jl:120-220         Q4 heat: N, quadrature, unknowns, nodal error
  test/qmesh*.dat, test/mt3gen3*.dat  mesh fixtures (data files)
"""
import json
import os
import re
import sys

REF = os.environ.get("ELFEL_REFERENCE")
OUT = os.path.dirname(os.path.abspath(__file__))

NUM = r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?"


def read(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read()


def numbers(s):
    return [float(x) for x in re.findall(NUM, s)]


def julia_matrix(s):
    """Parse a Julia matrix literal body ('a b c\n d e f' or 'a b; c d')."""
    rows = [r for r in re.split(r"[;\n]", s) if re.search(NUM, r)]
    return [numbers(r) for r in rows]


def block_after(text, start, open_ch="[", close_ch="]"):
    """Return the bracketed block starting at the first open_ch at/after start."""
    i = text.index(open_ch, start)
    depth = 0
    for j in range(i, len(text)):
        if text[j] == open_ch:
            depth += 1
        elif text[j] == close_ch:
            depth -= 1
            if depth == 0:
                return text[i + 1:j], j + 1
    raise ValueError("unbalanced")


def assemblers():
    t = read("test/test_assemblers.jl")
    mod = t[t.index("module mmass0\n"):t.index("module mmass0a")]
    pos = mod.index("m = [")
    m1, pos = block_after(mod, pos)
    gi1, pos = block_after(mod, mod.index("gi =", pos))
    gj1, pos = block_after(mod, mod.index("gj =", pos))
    m2, pos = block_after(mod, mod.index("m = [", pos))
    gi2, pos = block_after(mod, mod.index("gi =", pos))
    gj2, pos = block_after(mod, mod.index("gj =", pos))
    B, pos = block_after(mod, mod.index("B = [", pos))
    return {
        "source": "test/test_assemblers.jl:6-34",
        "nrow": 7, "ncol": 7,
        "blocks": [
            {"m": julia_matrix(m1), "gi": [int(x) for x in numbers(gi1)], "gj": [int(x) for x in numbers(gj1)]},
            {"m": julia_matrix(m2), "gi": [int(x) for x in numbers(gi2)], "gj": [int(x) for x in numbers(gj2)]},
        ],
        "B": julia_matrix(B),
        "rtol": 1.0e-5,
    }


def feiterators():
    t = read("test/test_feiterators.jl")
    m1 = t[t.index("module mfeit1"):t.index("module mfeit2")]
    refc, _ = block_after(m1, m1.index("refc = ["))
    conn = [[int(x) for x in numbers(b)] for b in re.findall(r"\[([^\[\]]*)\]", refc)]
    refd, _ = block_after(m1, m1.index("refd ="))
    dofs_by_node = [int(x) for x in numbers(refd)]
    ebc = [int(x) for x in numbers(re.search(r"for i in \[([^\]]*)\]", m1).group(1))]
    m2 = t[t.index("module mfeit2"):t.index("module mfeit3")]
    A, _ = block_after(m2, m2.index("A = ["))
    m3 = t[t.index("module mfeit3"):t.index("module maggfeit1")]
    ref3, _ = block_after(m3, m3.index("ref = ["))
    dofs3 = [[int(x) for x in numbers(b)] for b in re.findall(r"\[([^\[\]]*)\]", ref3)]
    comps = [int(x) for x in numbers(re.search(r"eldofcomps\(it\) == \[([^\]]*)\]", m3).group(1))]
    return {
        "source": "test/test_feiterators.jl:21-71,88-119,140-172",
        "qmesh_conn": conn,
        "ebc_nodes": ebc,
        "scalar_dofnum_by_node": dofs_by_node,
        "scalar_ndofs": 12, "scalar_nunknowns_free": 12, "scalar_nunknowns_ebc": 8,
        "A": julia_matrix(A),
        "vec3_eldofs": dofs3,
        "vec3_eldofcomps": comps,
    }


def heat():
    t = read("test/test_heat.jl")
    m = t[t.index("module mt_heat_poisson_t3"):t.index("module m_heat_poisson_q4")]
    N = int(re.search(r"\nN = (\d+);", m).group(1))
    kappa = float(re.search(r"kappa =\s*(" + NUM + ")", m).group(1))
    Q = float(re.search(r"Q = (" + NUM + ")", m).group(1))
    vec, _ = block_after(m, m.index("@test isapprox(T, ["))
    return {
        "source": "test/test_heat.jl:22-26,78-87,110",
        "N": N, "A": 1.0, "kappa": kappa, "Q": Q,
        "T": numbers(vec),
        "mean_nodal_error_max": 1.0e-9,
    }


def stokes():
    t = read("test/test_stokes.jl")
    counts = re.search(r"@test \(tndof, tnunk\) == \((\d+), (\d+)\)", t)
    ms = t[t.index("module mstok1"):]
    refb, _ = block_after(ms, ms.index("ref = ["))
    pairs = [numbers(p) for p in re.findall(r"\(([^()]*)\)", refb)]
    alt = t[t.index("module m_th_p2_p1_veclap_alt\n"):]
    alt = alt[:alt.index("module m_th_p2_p1_veclap_alt_e")]
    altv = re.search(r"isapprox\(\[ep, ev\], \[([^\]]*)\]\)", alt).group(1)
    return {
        "source": "test/test_stokes.jl:25-27,130,551-558,777-780",
        "driven_cavity_N": 100,
        "driven_cavity_tndof_tnunk": [int(counts.group(1)), int(counts.group(2))],
        "reddy_th_errors": {"N": [4, 8, 16], "ep_ev": pairs},
        "veclap_th_errors": {"N": 4, "ep_ev": numbers(altv)},
    }


def qpiterators():
    t = read("test/test_qpiterators.jl")
    b1, pos = block_after(t, t.index("refNs = ["))
    b3, pos = block_after(t, t.index("refNs = [", pos))
    g, pos = block_after(t, t.index("refgNs = [", pos))
    w = float(re.search(r"@test w == (" + NUM + ")", t).group(1))
    t2 = read("test/test_refshapes.jl")
    m = t2[t2.index("module mrs2"):t2.index("module mrs3")]
    pc, _ = block_after(m, m.index("param_coords(qr), ["))
    wt, _ = block_after(m, m.index("weights(qr), ["))
    return {
        "source": "test/test_qpiterators.jl:22-61, test/test_refshapes.jl:26-29",
        "t3_1pt_N": [numbers(r) for r in re.findall(r"\[([^\[\]]*)\]", b1)],
        "t3_3pt_N": [numbers(r) for r in re.findall(r"\[([^\[\]]*)\]", b3)],
        "t3_gradpar": [numbers(r) for r in re.findall(r"\[([^\[\]]*)\]", g)],
        "weight_3pt": w,
        "tri3_param_coords": julia_matrix(pc),
        "tri3_weights": numbers(wt),
    }


def fefields():
    t = read("test/test_fefields.jl")
    return {
        "source": "test/test_fefields.jl:13-52",
        "ndofsperterm": 2,
        "ebc": [[3, 2, 3.0], [5, 1, 5.0]],
        "highest_free_no_ebc": int(re.search(r"highestfreedofnum\(fef\) == (\d+)", t).group(1)),
        "highest_free_ebc": 40, "highest_data_ebc": 42,
    }


def _module(text, name):
    start = text.index("module " + name + "\n")
    end = text.find("\nmodule ", start + 8)
    return text[start:end if end >= 0 else len(text)]


def _after(text, anchor):
    """Body of the first bracketed literal after anchor."""
    body, _ = block_after(text, text.index(anchor) + len(anchor))
    return body


def terms(s):
    """Comma/space separated literal terms, each a number or a product or
    quotient of numbers (e.g. '2*0.3333', '1/4')."""
    out = []
    for t in re.split(r"[,\s;]+", s.strip()):
        if not t:
            continue
        if not re.fullmatch(r"[-+0-9.eE*/]+", t):
            raise ValueError(t)
        v = None
        for k, part in enumerate(re.split(r"([*/])", t)):
            if k == 0:
                v = float(part)
            elif k % 2 == 1:
                op = part
            else:
                v = v * float(part) if op == "*" else v / float(part)
        out.append(v)
    return out


def elements():
    rs = read("test/test_refshapes.jl")
    m1, m3, m5 = _module(rs, "mrs1"), _module(rs, "mrs3"), _module(rs, "mrs5")
    m6, m7 = _module(rs, "mrs6"), _module(rs, "mrs7")
    tet = []
    pos = 0
    for _ in range(3):
        n = int(re.search(r"@test npts\(qr\) == (\d+)", m6[pos:]).group(1))
        pc, pos = block_after(m6, m6.index("param_coords(qr),", pos) + len("param_coords(qr),"))
        wt, pos = block_after(m6, m6.index("weights(qr),", pos) + len("weights(qr),"))
        tet.append({"npts": n, "param_coords": julia_matrix(pc), "weights": terms(wt)})
    fe = read("test/test_felements.jl")
    f1 = _module(fe, "mfes1")
    l2 = f1[f1.index("fe = FEH1_L2()"):]
    f2 = _module(fe, "mfes2")
    counts = {}
    for mod in ("mfes2", "mfes3", "mfes4"):
        parts = re.split(r"fe = (FE\w+)\(\)", _module(fe, mod))[1:]
        for k in range(0, len(parts), 2):
            body = parts[k + 1]
            counts[parts[k]] = {
                "nfeatofdim": [int(x) for x in re.findall(r"nfeatofdim\(fe, \d\) == (\d+)", body)],
                "ndofperfeat": [int(x) for x in re.findall(r"ndofperfeat\(fe, \d\) == (\d+)", body)],
                "bfun": terms(_after(body, "isapprox(bfun(fe, [" + body.split("isapprox(bfun(fe, [")[1].split("]")[0]
                                     + "]),")),
            }
    fs = read("test/test_fespaces.jl")
    fb = fs[fs.index("FESpace(Float64, mesh, FEH1_T3_BUBBLE(), 1)"):]
    fb = fb[:fb.index("FESpace(Float64, mesh, FEH1_T3_BUBBLE(), 2)")]
    ht = read("test/test_heat.jl")
    hq = ht[ht.index("module m_heat_poisson_q4"):]
    return {
        "source": "test/test_refshapes.jl, test/test_felements.jl, test/test_fespaces.jl:85-172, "
                  "test/test_heat.jl:120-220",
        "interval_default_npts": int(re.search(r"@test npts\(qr\) == (\d+)", m1).group(1)),
        "interval_order3": {"param_coords": terms(_after(m1, "param_coords(qr),")),
                            "weights": terms(_after(m1, "weights(qr),"))},
        "square_order2_point3": terms(_after(m3, "param_coords(qr)[3, :]),")),
        "square_orders": [int(x) for x in re.search(r"for o in (\d+):(\d+)", _module(rs, "mrs4")).groups()],
        "triangle_npts": [int(x) for x in re.search(r"for n in \[([^\]]*)\]", m5).group(1).split(",")],
        "tetrahedron": tet,
        "interval_exp_integrals": terms(_after(m7, "reference_results =")),
        "L2": {"bfun_at_one_third": terms(_after(l2, "bfun(fe, [1/3]),")),
               "gradpar": [terms(_after(l2, "g[1],")), terms(_after(l2, "g[2],"))]},
        "T4_gradpar": [terms(b) for b in re.findall(r"isapprox\(g\[\d\], \[([^\]]*)\]", f2)],
        "counts": counts,
        "bubble": {"nfeatofdim": [int(x) for x in re.findall(r"nfeatofdim\(fesp.fe, \d\) == (\d+)", fb)],
                   "ndofperfeat": [int(x) for x in re.findall(r"ndofperfeat\(fesp.fe, \d\) == (\d+)", fb)],
                   "ndofsperel": int(re.search(r"ndofsperel\(fesp.fe\) == (\d+)", fb).group(1)),
                   "bfun_at_one_third": terms(_after(fb, "bfun(fesp.fe, [1/3, 1/3]),"))},
        "heat_q4": {"N": int(re.search(r"\nN = (\d+);", hq).group(1)),
                    "order": int(re.search(r"kind = :Gauss, order = (\d+)", hq).group(1)),
                    "nunknowns": int(re.search(r"nunknowns\(fesp\) == (\d+)", hq).group(1)),
                    "kappa": float(re.search(r"kappa =\s*(" + NUM + ")", hq).group(1)),
                    "Q": float(re.search(r"Q = (" + NUM + ")", hq).group(1)),
                    "mean_nodal_error_max": float(re.search(r"<= (" + NUM + ")", hq).group(1))},
    }


def datfile(rel):
    return [numbers(line) for line in read(rel).splitlines() if line.strip()]


def main():
    if not REF:
        sys.exit("set ELFEL_REFERENCE to a checkout of the reference project (Elfel.jl v0.4.0)")
    if not os.path.isdir(REF):
        sys.exit(f"reference not found at {REF}")
    out = {
        "assemblers.json": assemblers(),
        "feiterators.json": feiterators(),
        "heat_t3.json": heat(),
        "stokes.json": stokes(),
        "qpiterators.json": qpiterators(),
        "fefields.json": fefields(),
        "elements.json": elements(),
        "meshes.json": {
            "source": "test/qmesh-xyz.dat, test/qmesh-conn.dat, test/mt3gen3-xyz.dat, test/mt3gen3-conn.dat",
            "qmesh_xyz": datfile("test/qmesh-xyz.dat"),
            "qmesh_conn": [[int(x) for x in r] for r in datfile("test/qmesh-conn.dat")],
            "mt3gen3_xyz": datfile("test/mt3gen3-xyz.dat"),
            "mt3gen3_conn": [[int(x) for x in r] for r in datfile("test/mt3gen3-conn.dat")],
        },
    }
    # test_fefields.jl asserts highestfreedofnum 40 and highestdatadofnum 42 with
    # two EBCs; check that these literals are present in the source.
    t = read("test/test_fefields.jl")
    assert "highestfreedofnum(fef) == 40" in t and "highestdatadofnum(fef) == 42" in t
    for name, obj in out.items():
        with open(os.path.join(OUT, name), "w") as f:
            json.dump(obj, f, indent=1)
        print("wrote", name)


if __name__ == "__main__":
    main()
