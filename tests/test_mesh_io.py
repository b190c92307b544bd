"""gmsh v2.2 reader (ia_read_msh, host code in libia.so) against the
reference's own geometry() output frozen in tests/golden (CUDA/utils.cuh:291),
and the oracle's restatement of it.  No GPU needed."""
import os

import numpy as np
import pytest

from oracle import ia_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
MSH = os.path.join(HERE, "golden", "sphere42.msh")


def test_oracle_reader_matches_reference(golden):
    n, f, e = O.read_msh(MSH, float(golden["msh_k"]), float(golden["msh_t"]))
    assert np.array_equal(n, golden["msh_nodes"])
    assert np.array_equal(f, golden["msh_field"])
    assert np.array_equal(e, golden["msh_elems"])


def test_library_reader_matches_reference(golden):
    from inverseacoustics_gb300 import api
    n, f, e = api.read_msh(MSH, float(golden["msh_k"]), float(golden["msh_t"]))
    assert np.array_equal(n, golden["msh_nodes"])
    assert np.array_equal(f, golden["msh_field"])
    assert np.array_equal(e, golden["msh_elems"])
    assert e.shape[1] == golden["mesh_elems"].shape[1]          # degenerate triangles and points dropped


def test_reader_errors_and_variants(tmp_path, golden):
    from inverseacoustics_gb300 import api
    from inverseacoustics_gb300._lib import IAError
    with pytest.raises(IAError) as ei:
        api.read_msh(str(tmp_path / "missing.msh"), 1.0)
    assert ei.value.code == 1
    bad = tmp_path / "bad.msh"
    bad.write_text("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n3\n1 0 0\n")
    with pytest.raises(IAError):
        api.read_msh(str(bad), 1.0)
    # CR-LF line ends and three tags per element (the reference assumes two)
    text = open(MSH).read()
    lines = text.split("\n")
    out = []
    in_el = False
    for s in lines:
        if s == "$Elements":
            in_el = True
        elif s == "$EndElements":
            in_el = False
        elif in_el and len(s.split()) > 3:
            f = s.split()
            f[2] = str(int(f[2]) + 1)
            f.insert(3 + int(f[2]) - 1, "7")
            s = " ".join(f)
        out.append(s)
    var = tmp_path / "crlf3.msh"
    var.write_bytes("\r\n".join(out).encode())
    n, f, e = api.read_msh(str(var), float(golden["msh_k"]), float(golden["msh_t"]))
    assert np.array_equal(n, golden["msh_nodes"]) and np.array_equal(e, golden["msh_elems"])
