"""Extract the known-answer data of the reference's own tests into JSON.

Run with the path of a FinEtools.jl source checkout, as an argument or in
the FINETOOLS_REF environment variable (one of them is required):

    python tests/golden/make_golden.py <path of the FinEtools.jl sources>

It reads the Julia test files as text (nothing is executed), pulls out the
literal matrices, DOF lists, mesh parameters and expected answers of the
assembly-path tests, and writes ``tests/golden/reference_kats.json``.  The
JSON is committed so that the tests never need the reference sources.
"""
from __future__ import annotations

import json
import os
import re
import sys

REF = None  # the FinEtools.jl source checkout (command line or FINETOOLS_REF)
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")


def read(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read()


def module_text(src, name, rel):
    """Text of `module <name>` up to the next top-level `module`."""
    m = re.search(r"^module %s\s*$" % re.escape(name), src, re.M)
    if not m:
        raise KeyError(f"module {name} not found in {rel}")
    nxt = re.search(r"^module \w+", src[m.end():], re.M)
    end = m.end() + nxt.start() if nxt else len(src)
    line = src[: m.start()].count("\n") + 1
    return src[m.start():end], line


def parse_matrix(text, start):
    """Parse the Julia matrix literal whose '[' is at text[start]."""
    assert text[start] == "["
    depth, i = 0, start
    while True:
        if text[i] == "[":
            depth += 1
        elif text[i] == "]":
            depth -= 1
            if depth == 0:
                break
        i += 1
    body = text[start + 1: i]
    rows = [r for r in re.split(r"[;\n]", body) if r.strip()]
    mat = [[float(x) for x in r.split()] for r in rows]
    return mat, i + 1


def matrices_after(text, anchor_regex):
    out = []
    for m in re.finditer(anchor_regex, text):
        j = text.index("[", m.end() - 1)
        mat, _ = parse_matrix(text, j)
        out.append(mat)
    return out


def int_list(s):
    return [int(x) for x in re.findall(r"-?\d+", s)]


def assembler_kats():
    kats = {}
    rel = "test/test_miscellaneous.jl"
    src = read(rel)
    # SysmatAssemblerSparse: two rectangular matrices into 7x7
    txt, line = module_text(src, "mmassembly", rel)
    ms = matrices_after(txt, r"\bm = \[")
    asm = re.findall(r"assemble!\(a, m, \[([^\]]*)\], \[([^\]]*)\]\)", txt)
    expected = matrices_after(txt, r"maximum\(\s*\[")
    kats["sparse_rect"] = {
        "source": f"{rel}:{line}", "kind": "sparse", "size": 7,
        "mats": ms, "rows": [int_list(a) for a, _ in asm], "cols": [int_list(b) for _, b in asm],
        "expected": expected[0],
    }
    txt, line = module_text(src, "mmassembly2", rel)
    ms = matrices_after(txt, r"\bm = \[")
    asm = re.findall(r"assemble!\(a, m' \* m, \[([^\]]*)\], \[([^\]]*)\]\)", txt)
    expected = matrices_after(txt, r"maximum\(\s*\[")
    kats["symm_mtm"] = {
        "source": f"{rel}:{line}", "kind": "symm", "size": 7, "form": "mtm",
        "mats": ms, "rows": [int_list(a) for a, _ in asm], "cols": [int_list(b) for _, b in asm],
        "expected": expected[0],
    }
    rel = "test/test_basics.jl"
    src = read(rel)
    txt, line = module_text(src, "mmassembly2ya1", rel)
    m1 = matrices_after(txt, r"\bm1 = \[")[0]
    m2 = matrices_after(txt, r"\bm2 = \[")[0]
    i1 = int_list(re.search(r"i1 = vec\(\[([^\]]*)\]\)", txt).group(1))
    i2 = int_list(re.search(r"i2 = vec\(\[([^\]]*)\]\)", txt).group(1))
    testA = matrices_after(txt, r"testA = \[")[0]
    kats["sparse_and_symm_mtm"] = {
        "source": f"{rel}:{line}", "size": 7, "form": "mtm",
        "mats": [m1, m2], "dofs": [i1, i2], "expected": testA,
    }
    txt, line = module_text(src, "mmassembly2ya2", rel)
    m1 = matrices_after(txt, r"\bm1 = \[")[0]
    m2 = matrices_after(txt, r"\bm2 = \[")[0]
    i1 = int_list(re.search(r"i1 = vec\(\[([^\]]*)\]\)", txt).group(1))
    i2 = int_list(re.search(r"i2 = vec\(\[([^\]]*)\]\)", txt).group(1))
    testA = matrices_after(txt, r"testA = \[")[0]
    kats["sparse_diag_mtm"] = {
        "source": f"{rel}:{line}", "kind": "diag", "size": 7, "form": "mtm",
        "mats": [m1, m2], "dofs": [i1, i2], "expected": testA,
    }
    txt, line = module_text(src, "massnomat1", rel)
    ms = matrices_after(txt, r"\bm = \[")
    asm = re.findall(r"assemble!\(a, m, \[([^\]]*)\], \[([^\]]*)\]\)", txt)
    spots = [(int(r), int(c), float(v)) for r, c, v in
             re.findall(r"A\[(\d+), (\d+)\] ≈ ([0-9.]+)", txt)]
    kats["nomatrixresult"] = {
        "source": f"{rel}:{line}", "kind": "sparse", "size": 7, "mats": ms,
        "rows": [int_list(a) for a, _ in asm], "cols": [int_list(b) for _, b in asm],
        "spots": spots,
    }
    return kats


def num(txt, name):
    m = re.search(r"\b%s = ([-0-9.e/]+)" % re.escape(name), txt)
    v = m.group(1)
    if "/" in v:
        a, b = v.split("/")
        return float(a) / float(b)
    return float(v)


def tuple_vals(txt, names):
    m = re.search(r"%s = \(?([^)\n]*)\)?" % re.escape(names), txt)
    vals = []
    for v in m.group(1).split(","):
        v = v.strip()
        if "/" in v:
            a, b = v.split("/")
            vals.append(float(a) / float(b))
        else:
            vals.append(float(v))
    return vals


def block_args(txt, fn):
    """Arguments of `fn(L, W, t, nl, nw, nt)` mapped through the local names."""
    m = re.search(r"%s\(([^)]*)\)" % re.escape(fn), txt)
    return [a.strip() for a in m.group(1).split(",")]


def patch_tests():
    rel = "test/test_forms.jl"
    src = read(rel)
    out = []
    specs = [
        ("mbilform_dot_1", "dot_volume", "H8block", 2),
        ("mbilform_diffusion_1", "diffusion_constant_field", "H8block", 2),
        ("mbilform_diffusion_2", "diffusion_linear_field", "H8block", 2),
        ("mbilform_diffusion_3", "diffusion_linear_field", "H20block", 3),
        ("mdistributedl1x", "distribloads_sum", "H8block", 2),
        ("mbilform_lin_elastic_1", "elastic_rigid_translation", "H8block", 2),
        ("mbilform_lin_elastic_2", "elastic_linear_field", "H8block", 2),
        ("mbilform_div_grad_5", "elastic_symmetry_linear_field", "H8block", 2),
    ]
    for mod, kind, gen, order in specs:
        txt, line = module_text(src, mod, rel)
        W, L, t = num(txt, "W"), num(txt, "L"), num(txt, "t")
        sizes = dict(zip(["nl", "nt", "nw"], tuple_vals(txt, "nl, nt, nw")))
        args = block_args(txt, gen)
        env = {"W": W, "L": L, "t": t, **sizes}
        rec = {"source": f"{rel}:{line}", "module": mod, "kind": kind, "generator": gen,
               "block": [env[a] for a in args[:3]] + [int(env[a]) for a in args[3:6]],
               "gauss_order": order, "volume": W * L * t, "tol": 1.0e-5}
        if "a, b, c, d" in txt:
            rec["abcd"] = tuple_vals(txt, "a, b, c, d")
        if re.search(r"\bmu = ", txt):
            rec["mu"] = num(txt, "mu")
        if "u_x, u_y, u_z" in txt:
            rec["uxyz"] = tuple_vals(txt, "u_x, u_y, u_z")
        if kind == "distribloads_sum":
            rec["force"] = 11.0
            rec["norm"] = 667.0
        out.append(rec)
    rel = "test/test_basics.jl"
    src = read(rel)
    txt, line = module_text(src, "mgram1a", rel)
    W, L, t = num(txt, "W"), num(txt, "L"), num(txt, "t")
    sizes = dict(zip(["nl", "nt", "nw"], tuple_vals(txt, "nl, nt, nw")))
    args = block_args(txt, "H8block")
    env = {"W": W, "L": L, "t": t, **sizes}
    out.append({"source": f"{rel}:{line}", "module": "mgram1a", "kind": "dot_volume_3dof",
                "generator": "H8block", "block": [env[a] for a in args[:3]] +
                [int(env[a]) for a in args[3:6]], "gauss_order": 2, "volume": W * L * t,
                "tol": 1.0e-5})
    return out


def coloring_and_pattern():
    rel = "test/test_meshing.jl"
    src = read(rel)
    out = {}
    for gen, key in (("H8block", "h8"), ("T4block", "t4")):
        for m in re.finditer(r"fens, fes = %s\(W, L, H, N, N, N\)" % gen, src):
            seg = src[m.start(): m.start() + 1500]
            exp = re.search(r"unique\(coloring\[1\]\) - \[([^\]]*)\]", seg)
            if not exp:
                continue
            head = src[max(0, m.start() - 400): m.start()]
            line = src[: m.start()].count("\n") + 1
            out[f"coloring_{key}"] = {
                "source": f"{rel}:{line}", "generator": gen,
                "block": [num(head, "W"), num(head, "L"), num(head, "H")] + [int(num(head, "N"))] * 3,
                "unique_colors_in_order": int_list(exp.group(1)),
            }
    rel = "test/test_miscellaneous.jl"
    src = read(rel)
    txt, line = module_text(src, "mmconnection1", rel)
    h = 0.05
    out["connection_degree"] = {
        "source": f"{rel}:{line}", "generator": "H8block",
        "block": [h, 10 * h, 2.0 * 3.141592653589793, int(num(txt, "nh")), int(num(txt, "nl")),
                  int(num(txt, "nc"))],
        "max_degree": int(re.search(r"maximum\(Degree\) == (\d+)", txt).group(1)),
        "min_degree": int(re.search(r"minimum\(Degree\) == (\d+)", txt).group(1)),
    }
    return out


def cg_case():
    """The system of the conjugategradient test (test/test_miscellaneous.jl,
    module mconjugategradient1): A, b, x0 = 0 and maxiter."""
    rel = "test/test_miscellaneous.jl"
    txt, line = module_text(read(rel), "mconjugategradient1", rel)
    A, _ = parse_matrix(txt, txt.index("[", re.search(r"A\s*=", txt).end()))
    b, _ = parse_matrix(txt, txt.index("[", re.search(r"\bb\s*=", txt).end()))
    maxiter = int(re.search(r"maxiter\s*=\s*(\d+)", txt).group(1))
    return {"source": f"{rel}:{line}", "A": A, "b": [r[0] for r in b], "maxiter": maxiter}


def div_grad_cases():
    """bilform_div_grad identities (test/test_forms.jl, modules
    mbilform_div_grad_1..3): a constant velocity has no energy, a linear one
    the energy 2 mu V |sym grad u|^2, and for any field the energy equals the
    elasticity energy with C = diag(2mu, 2mu, 2mu, mu, mu, mu)."""
    rel = "test/test_forms.jl"
    src = read(rel)
    out = []
    for mod, kind in (("mbilform_div_grad_1", "constant_field"),
                      ("mbilform_div_grad_2", "linear_field"),
                      ("mbilform_div_grad_3", "vs_elastic")):
        txt, line = module_text(src, mod, rel)
        W, L, t = num(txt, "W"), num(txt, "L"), num(txt, "t")
        sizes = dict(zip(["nl", "nt", "nw"], tuple_vals(txt, "nl, nt, nw")))
        args = block_args(txt, "H8block")
        env = {"W": W, "L": L, "t": t, **sizes}
        rec = {"source": f"{rel}:{line}", "module": mod, "kind": kind,
               "block": [env[a] for a in args[:3]] + [int(env[a]) for a in args[3:6]],
               "gauss_order": int(re.search(r"GaussRule\(3,\s*(\d+)\)", txt).group(1)),
               "volume": W * L * t, "mu": num(txt, "mu"), "tol": 1.0e-5}
        if "u_x, u_y, u_z" in txt:
            rec["uxyz"] = tuple_vals(txt, "u_x, u_y, u_z")
        if "a, b, c, d" in txt:
            rec["abcd"] = tuple_vals(txt, "a, b, c, d")
        out.append(rec)
    return out


def ffblock_case():
    """SysmatAssemblerFFBlock against matrix_blocked_ff (test/test_forms.jl,
    module mbilform_diffusion_assembly_1): the block mesh, the nodes whose DOF
    is fixed, and the tolerance."""
    rel = "test/test_forms.jl"
    txt, line = module_text(read(rel), "mbilform_diffusion_assembly_1", rel)
    W, L, t = num(txt, "W"), num(txt, "L"), num(txt, "t")
    sizes = dict(zip(["nl", "nt", "nw"], tuple_vals(txt, "nl, nt, nw")))
    args = block_args(txt, "H8block")
    env = {"W": W, "L": L, "t": t, **sizes}
    fixed = re.search(r"nl = collect\((\d+):(\d+)\)", txt)
    return {"source": f"{rel}:{line}",
            "block": [env[a] for a in args[:3]] + [int(env[a]) for a in args[3:6]],
            "gauss_order": int(re.search(r"GaussRule\(3,\s*(\d+)\)", txt).group(1)),
            "fixed_nodes": list(range(int(fixed.group(1)), int(fixed.group(2)) + 1)),
            "tol": 1.0e-5}


def axisymmetric_case():
    """Volume of an axisymmetric domain (test/test_basics.jl, module
    mbas010x1): the rectangle a x b revolved about the axis has volume
    pi a^2 b."""
    rel = "test/test_basics.jl"
    txt, line = module_text(read(rel), "mbas010x1", rel)
    a, b, na, nb = tuple_vals(txt, "a, b, na, nb")
    order = int(re.search(r"GaussRule\(2,\s*(\d+)\)", txt).group(1))
    return {"source": f"{rel}:{line}", "a": a, "b": b, "na": int(na), "nb": int(nb),
            "gauss_order": order}


def masslike_case():
    """bilform_masslike known answer (test/test_forms.jl, module
    mbilform_masslike_1): the L2 mesh's node coordinates, the Gauss order and
    the expected dense matrix."""
    rel = "test/test_forms.jl"
    txt, line = module_text(read(rel), "mbilform_masslike_1", rel)
    vec = lambda name: [float(x) for x in re.search(name + r"\s*=\s*\[([^\]]*)\]", txt)
                        .group(1).split(",")]
    order = int(re.search(r"GaussRule\(1,\s*(\d+)\)", txt).group(1))
    G, _ = parse_matrix(txt, txt.index("[", re.search(r"Matrix\(G\)\s*==", txt).end()))
    return {"source": f"{rel}:{line}", "xs": vec("xs"), "ys": vec("ys"), "gauss_order": order,
            "G": G}


def main():
    global REF
    REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FINETOOLS_REF")
    if not REF:
        sys.exit("usage: make_golden.py <path of the FinEtools.jl sources> "
                 "(or set FINETOOLS_REF)")
    if not os.path.isdir(REF):
        sys.exit(f"reference sources not found at {REF}")
    data = {"assembler": assembler_kats(), "patch": patch_tests(), **coloring_and_pattern(),
            "conjugategradient": cg_case(), "masslike": masslike_case(),
            "div_grad": div_grad_cases(), "ffblock": ffblock_case(),
            "axisymmetric": axisymmetric_case()}
    with open(OUT, "w") as f:
        json.dump(data, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
