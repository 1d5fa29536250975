"""Host side of the serving engine (no GPU): request layout and the
footprint estimate used for admission."""
import ctypes

import numpy as np


def test_footprint_estimate_grows_with_size_and_degree():
    from modfem_gb300.mesh import prism_faces, structured_prism_mesh
    from modfem_gb300.serve import DG, STD, Problem
    fp = {}
    for n in (3, 6):
        m = structured_prism_mesh(n)
        k = np.ones(m.nel)
        F = prism_faces(m)
        fp[(n, "std")] = Problem(m, k, kind=STD).footprint()
        fp[(n, 1)] = Problem(m, k, kind=DG, p=1, faces=F).footprint()
        fp[(n, 2)] = Problem(m, k, kind=DG, p=2, faces=F).footprint()
    for n in (3, 6):
        assert 0 < fp[(n, "std")] < fp[(n, 1)] < fp[(n, 2)]
    assert fp[(6, "std")] > fp[(3, "std")] and fp[(6, 2)] > fp[(3, 2)]
    # DG p = 2 stores (18 / 6)^2 = 9 times the p = 1 values: the estimate follows
    assert fp[(6, 2)] > 4 * fp[(6, 1)]


def test_request_struct_matches_the_c_layout(tmp_path):
    """ctypes mirror of gbfem_serve_request against the C compiler's layout."""
    import os
    import shutil
    import subprocess
    import pytest
    from modfem_gb300.serve import Request
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    names = [f[0] for f in Request._fields_]
    src = tmp_path / "layout.c"
    src.write_text("#include <stddef.h>\n#include <stdio.h>\n#include \"modfem_gb300.h\"\nint main(void){\n"
                   + "".join(f'printf("%zu\\n", offsetof(gbfem_serve_request, {n}));\n' for n in names)
                   + 'printf("%zu\\n", sizeof(gbfem_serve_request));return 0;}\n')
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-I", os.path.join(root, "include"), str(src), "-o", str(exe)])
    got = [int(v) for v in subprocess.check_output([str(exe)]).split()]
    want = [getattr(Request, n).offset for n in names] + [ctypes.sizeof(Request)]
    assert got == want
