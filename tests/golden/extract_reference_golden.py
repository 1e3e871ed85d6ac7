"""Extract the reference's own golden vectors for the hot path into JSON.

Reads QMCPACK's unit-test sources as text (no reference code is built or run)
and writes tests/golden/reference_golden.json.  The committed JSON is what the
tests use; this script documents where every number comes from.

usage: python tests/golden/extract_reference_golden.py [REFERENCE_ROOT]
"""
import json
import os
import re
import sys

NUM = r"[-+]?\d*\.?\d+(?:[eE][-+]?\d+)?"


def read(root, rel):
    with open(os.path.join(root, rel)) as f:
        return f.read()


def block(text, start_pat, end_pat):
    i = text.index(start_pat)
    j = text.index(end_pat, i)
    return text[i:j]


def checks(text, lhs_pat):
    """All `CHECK(<lhs> == Approx(<num>))` with lhs matching lhs_pat, in order."""
    out = []
    for m in re.finditer(r"CHECK\((" + lhs_pat + r")\s*==\s*Approx\((" + NUM + r")\)", text):
        out.append((m.group(1).strip(), float(m.group(2))))
    return out


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("QMCPACK_REFERENCE_DIR", "/root/reference")
    g = {"source": "QMCPACK unit tests (read as text)"}

    # --- spline2 prefactors and VGH: src/spline2/tests/test_multi_spline.cpp
    rel = "src/spline2/tests/test_multi_spline.cpp"
    t = read(root, rel)
    pre = block(t, "void test_prefactors()", "TEST_CASE(\"double prefactors\"")
    tx = [float(x) for x in re.findall(r"tx = (" + NUM + r");", pre)]
    vals = checks(pre, r"d?2?a\[\d\]")
    g["prefactors"] = {"file": rel, "tx": tx, "checks": vals}
    spl = block(t, "struct test_splines<T, 5, 1>", "MultiBsplineOffloadMapper<T> mapped_bs(bs);")
    g["spline_vgh"] = {
        "file": rel,
        "grid": 5,
        "data": "sin(2 pi x) + sin(6 pi y) + sin(8 pi z) on the 5^3 periodic unit grid",
        "pos0": [0.0, 0.0, 0.0],
        "pos1": [0.1, 0.2, 0.3],
        "checks": checks(spl, r"v\[0\]|dv\[0\]\[\d\]|hess\[0\]\[\d\]|lap\[0\]\[0\]"),
    }

    # --- J2 B-spline functor: src/QMCWaveFunctions/tests/test_J2_bspline.cpp
    rel = "src/QMCWaveFunctions/tests/test_J2_bspline.cpp"
    t = read(root, rel)
    first = block(t, "TEST_CASE(\"BSpline builder Jastrow J2\"", "TEST_CASE(\"BSpline builder Jastrow J2 ")\
        if "TEST_CASE(\"BSpline builder Jastrow J2 " in t else t
    coefs = re.search(r'<coefficients id="ud" type="Array">([^<]+)</coefficients>', first).group(1).split()
    rcut = float(re.search(r'correlation rcut="(' + NUM + r')" size="(\d+)"', first).group(1))
    table = re.findall(r"\{(" + NUM + r"),\s*(" + NUM + r"),\s*(" + NUM + r"),\s*(" + NUM + r")\}", first)
    g["j2_functor"] = {
        "file": rel,
        "rcut": rcut,
        "cusp_ud": -0.5,
        "params": [float(c) for c in coefs],
        "table_r_u_du_ddu": [[float(x) for x in row] for row in table],
        "logpsi_r1": checks(first, r"logpsi_real")[0][1],
        "KE": checks(first, r"KE")[0][1],
        "elec": [[1.0, 0.0, 0.0], [0.0, 0.0, 0.0]],
        "newpos": [0.3, 0.2, 0.5],
        "ratio_0": checks(first, r"std::real\(ratio_0\)")[0][1],
        "ratio_1": checks(first, r"std::real\(ratio_1\)")[0][1],
        "log_after_accept_1": checks(first, r"std::real\(j2->get_log_value\(\)\)")[0][1],
    }

    # --- distance table PBC: src/Particle/tests/test_distance_table.cpp
    rel = "src/Particle/tests/test_distance_table.cpp"
    t = read(root, rel)
    b = block(t, "void test_distance_pbc_z_batched_APIs", "} // test_distance_pbc_z_batched_APIs")
    g["distance_pbc"] = {
        "file": rel,
        "cell": 6.0,
        "elec": [[0.0, 0.0, 0.0], [3.0, 0.0, 0.0], [0.0, 0.0, 3.0]],
        "shift0": [0.1, 0.2, -0.1],
        "disp": [0.2, 0.1, 0.3],
        "checks": checks(b, r"ee_dtable\.getDistRow\(1\)\[0\]|ee_dtable\.getDisplRow\(1\)\[0\]\[\d\]"),
    }

    # --- determinant with FakeSPO: src/QMCWaveFunctions/tests/{FakeSPO.cpp,test_DiracDeterminantBatched.cpp}
    rel = "src/QMCWaveFunctions/tests/FakeSPO.cpp"
    t = read(root, rel)

    def mat(name, n):
        m = [[0.0] * n for _ in range(n)]
        for i, j, v in re.findall(name + r"\((\d), (\d)\) = (" + NUM + r");", t):
            m[int(i)][int(j)] = float(v)
        return m

    a = mat(r"\ba", 3)
    a2 = mat(r"\ba2", 4)
    v2 = mat(r"\bv2", 4)
    v = [float(x) for x in re.findall(r"\bv\[\d\] = (" + NUM + r");", t)]
    gv = [[float(x) for x in m] for m in
          re.findall(r"gv\[\d\] = TinyVector<Value, DIM>\((" + NUM + r"), (" + NUM + r"), (" + NUM + r")\);", t)]
    rel2 = "src/QMCWaveFunctions/tests/test_DiracDeterminantBatched.cpp"
    t2 = read(root, rel2)
    first = block(t2, "void test_DiracDeterminantBatched_first()", "TEST_CASE(\"DiracDeterminantBatched_first\"")
    bs = []
    for chunk in first.split("checkMatrix(b, ddb.get_psiMinv())")[:2]:
        m = [[0.0] * 3 for _ in range(3)]
        for i, j, val in re.findall(r"b\((\d), (\d)\) = (" + NUM + r");", chunk):
            m[int(i)][int(j)] = float(val)
        bs.append(m)
    g["det_fakespo"] = {
        "file": [rel, rel2],
        "a": a, "v": v, "a2": a2, "v2": v2, "gv": gv,
        "b_initial": bs[0],
        "b_after_accept0": bs[1],
        "det_ratio_0": float(re.search(r"det_ratio1 = (" + NUM + r");", first).group(1)),
        "ratio_1": checks(first, r"std::real\(ratio_1\)")[0][1],
        "log_after_accept_1": checks(first, r"std::real\(ddb.get_log_value\(\)\)")[0][1],
    }

    # --- standalone Ewald sums: src/QMCHamiltonians/tests/test_EwaldRef.cpp
    rel = "src/QMCHamiltonians/tests/test_EwaldRef.cpp"
    t = read(root, rel)
    cases = []
    for sec in re.split(r"SECTION\(", t)[1:]:
        name = re.match(r'"([^"]+)"', sec).group(1)
        A = [float(x) for x in re.search(r"A = \{([^}]+)\};", sec).group(1).split(",")]
        n = int(re.search(r"num_centers = (\d+);", sec).group(1))
        q0 = float(re.search(r"Q\.resize\(num_centers, (" + NUM + r")\);", sec).group(1))
        Q = [q0] * n
        loop = re.search(r"for \(int i = 0; i < (\d+); i\+\+\)\s*Q\[i\] = (" + NUM + r");", sec)
        if loop:
            for i in range(int(loop.group(1))):
                Q[i] = float(loop.group(2))
        R = [None] * n
        for i, x, y, z in re.findall(r"R\[(\d+)\]\s*= \{(" + NUM + r"), (" + NUM + r"), (" + NUM + r")\};", sec):
            R[int(i)] = [float(x), float(y), float(z)]
        assert all(r is not None for r in R)
        val = float(re.search(r"CHECK\(Approx\(Vii_ref\) == (" + NUM + r")\);", sec).group(1))
        cases.append({"name": name, "A": A, "Q": Q, "R": R, "energy": val})
    g["ewald_ref"] = {"file": rel, "approx_epsilon": 1.1920929e-05, "cases": cases}

    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_golden.json")
    with open(out, "w") as f:
        json.dump(g, f, indent=1)
    print("wrote", out)


if __name__ == "__main__":
    main()
