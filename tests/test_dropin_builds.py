"""The C++ drop-in (mara2_gb300/csrc/GpuSolutionScheme.hpp) compiles against
the reference's own interface headers and links against the reference's
hot-path objects and the CUDA library: a Mara2 driver can swap
MethodOfLinesTVD for GpuMethodOfLinesTVD.  Build only (no GPU here);
skipped where the reference tree is absent."""
import glob
import os
import subprocess

import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = os.environ.get("MARA_REF_SRC", os.path.join(ROOT, "baseline", "_ref", "src"))

DRIVER = r'''
#include "GpuSolutionScheme.hpp"
#include "SolutionSchemes.hpp"
// A regression driver's wiring (src/Problems.cpp:153-209) with the GPU scheme.
int main()
{
    auto cs = Cow::Shape {{128, 1, 1, 1, 1}};
    auto bs = Cow::Shape {{2, 0, 0, 0, 0}};
    auto mg = std::make_shared<CartesianMeshGeometry>();
    auto mo = std::make_shared<MeshOperator>();
    auto cl = std::make_shared<NewtonianHydro>();
    auto fs = std::make_shared<MethodOfLinesPlm>();
    auto fo = std::make_shared<FieldOperator>();
    auto md = std::make_shared<MeshData> (cs, bs, 5);
    auto bc = std::make_shared<OutflowBoundaryCondition>();
    mg->setCellsShape (cs);
    mo->setMeshGeometry (mg);
    fo->setConservationLaw (cl);
    GpuSchemeOptions opts;
    opts.gammaLawIndex = 1.4;
    auto ss = std::make_shared<GpuMethodOfLinesTVD> (opts);
    ss->setRungeKuttaOrder (2);
    ss->setFieldOperator (fo);
    ss->setMeshOperator (mo);
    ss->setBoundaryCondition (bc);
    ss->setIntercellFluxScheme (fs);
    std::shared_ptr<SolutionScheme> scheme = ss;
    if (scheme->getStencilSize() != 2) return 1;
    return 0;   // advance() needs a GPU; this program is only built
}
'''


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference tree not available")
def test_dropin_compiles_and_links(tmp_path):
    from mara2_gb300 import build
    lib = build.build()
    O.build(ref=True)
    objs = [o for o in glob.glob(os.path.join(ROOT, "oracle", "_ref", "obj", "*.o"))]
    src = tmp_path / "driver.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "driver"
    cmd = ["g++", "-std=c++14", "-O1", "-I" + os.path.join(ROOT, "oracle", "cowshim"), "-I" + REF_SRC,
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "mara2_gb300", "csrc"),
           str(src), *objs, "-L" + os.path.dirname(lib), "-lmara_gpu",
           "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert exe.exists()
