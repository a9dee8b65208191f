// A Mara2 driver with the GPU scheme swapped in (built by the tests against
// the reference's own headers and objects; not part of the library).
//
//   dropin_driver sod  <in> <out>   Sod 64 (regress-1d's wiring,
//       src/Problems.cpp:153-209): P0 and the dt sequence from <in>, each
//       step ss->advance(*md, 0.0, dt) as the drivers' advance lambda calls
//       it (Problems.cpp:188); P and the GPU Courant step of P0 to <out>
//   dropin_driver fail <in> <out>   an MHD 6^3 state that cannot be inverted:
//       advance must throw FieldOperator::InversionFailure; the first failed
//       zone to <out>
//   dropin_driver ct   <in> <out>   GpuConstrainedTransport (the
//       ConstrainedTransport interface): a cell field B (n0 n1 n2 then the
//       values) assigned, computeMonopole (vert, cell) and computeCurrent to
//       <out>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <vector>

#include "GpuSolutionScheme.hpp"
#include "SolutionSchemes.hpp"

static std::vector<double> read_doubles(const char* path)
{
    std::ifstream f(path, std::ios::binary);
    std::vector<double> v;
    double x;
    while (f.read(reinterpret_cast<char*>(&x), sizeof x)) v.push_back(x);
    return v;
}

static void write_doubles(const char* path, const double* p, size_t n)
{
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(p), n * sizeof(double));
}

static int run_sod(const char* in, const char* out)
{
    auto v = read_doubles(in);       // P0 (68 x 5), then the dts
    const int n = 64, ng = 2, nq = 5;
    const size_t cells = (size_t) (n + 2 * ng) * nq;
    auto cs = Cow::Shape {{n, 1, 1, 1, 1}};
    auto bs = Cow::Shape {{ng, 0, 0, 0, 0}};
    auto mg = std::make_shared<CartesianMeshGeometry>();
    auto mo = std::make_shared<MeshOperator>();
    auto cl = std::make_shared<NewtonianHydro>();
    auto fs = std::make_shared<MethodOfLinesPlm>();
    auto fo = std::make_shared<FieldOperator>();
    auto md = std::make_shared<MeshData> (cs, bs, nq);
    auto bc = std::make_shared<OutflowBoundaryCondition>();
    cl->setGammaLawIndex (1.4);
    mg->setCellsShape (cs);
    mo->setMeshGeometry (mg);
    fo->setConservationLaw (cl);
    fs->setPlmTheta (1.5);
    GpuSchemeOptions opts;
    opts.gammaLawIndex = 1.4;
    opts.riemannSolver = MARA_RIEMANN_HLLE;
    auto ss = std::make_shared<GpuMethodOfLinesTVD> (opts);
    ss->setRungeKuttaOrder (2);
    ss->setFieldOperator (fo);
    ss->setMeshOperator (mo);
    ss->setBoundaryCondition (bc);
    ss->setIntercellFluxScheme (fs);
    std::shared_ptr<SolutionScheme> scheme = ss;

    std::memcpy (md->P.data(), v.data(), cells * sizeof (double));
    const double dt0 = ss->getCourantTimestep (*md);
    auto advance = [&] (double dt) { scheme->advance (*md, 0.0, dt); };
    for (size_t k = cells; k < v.size(); ++k) advance (v[k]);
    std::vector<double> o (md->P.data(), md->P.data() + cells);
    o.push_back (dt0);
    write_doubles (out, o.data(), o.size());
    return 0;
}

static int run_fail(const char* in, const char* out)
{
    auto v = read_doubles(in);       // P (10^3 x 8)
    const int n = 6, ng = 2, nq = 8;
    auto cs = Cow::Shape {{n, n, n, 1, 1}};
    auto bs = Cow::Shape {{ng, ng, ng, 0, 0}};
    auto mg = std::make_shared<CartesianMeshGeometry>();
    auto mo = std::make_shared<MeshOperator>();
    auto cl = std::make_shared<NewtonianMHD>();
    auto fs = std::make_shared<MethodOfLinesPlm>();
    auto fo = std::make_shared<FieldOperator>();
    auto md = std::make_shared<MeshData> (cs, bs, nq);
    auto bc = std::make_shared<PeriodicBoundaryCondition>();
    mg->setCellsShape (cs);
    mo->setMeshGeometry (mg);
    fo->setConservationLaw (cl);
    GpuSchemeOptions opts;
    auto ss = std::make_shared<GpuMethodOfLinesTVD> (opts);
    ss->setRungeKuttaOrder (3);
    ss->setFieldOperator (fo);
    ss->setMeshOperator (mo);
    ss->setBoundaryCondition (bc);
    ss->setIntercellFluxScheme (fs);
    std::memcpy (md->P.data(), v.data(), v.size() * sizeof (double));
    double zone[4] = {-1, -1, -1, 0};
    try
    {
        ss->advance (*md, 0.0, 0.05);
    }
    catch (FieldOperator::InversionFailure& e)
    {
        // the zone the reference's message names ("at zone index [i j k]")
        int i = -1, j = -1, k = -1;
        std::sscanf (e.what(), "at zone index [%d %d %d]", &i, &j, &k);
        zone[0] = i;
        zone[1] = j;
        zone[2] = k;
        zone[3] = 1;
        std::printf ("InversionFailure: %s\n", e.what());
    }
    write_doubles (out, zone, 4);
    return 0;
}

static int run_ct(const char* in, const char* out)
{
    auto v = read_doubles(in);       // n0 n1 n2, then B (n0, n1, n2, 3)
    const int n0 = (int) v[0], n1 = (int) v[1], n2 = (int) v[2];
    auto mg = std::make_shared<CartesianMeshGeometry>();
    mg->setCellsShape (Cow::Shape {{n0, n1, n2, 1, 1}});
    auto ct = std::make_shared<GpuConstrainedTransport>();
    std::shared_ptr<ConstrainedTransport> iface = ct;
    iface->setMeshGeometry (mg);
    iface->setBoundaryCondition (std::make_shared<PeriodicBoundaryCondition>());
    auto B = Cow::Array (n0, n1, n2, 3);
    std::memcpy (B.data(), v.data() + 3, sizeof (double) * B.size());
    iface->assignCellCenteredB (B);
    auto Mv = iface->computeMonopole (MeshLocation::vert);
    auto Mc = iface->computeMonopole (MeshLocation::cell);
    auto J = iface->computeCurrent (MeshLocation::cell);
    std::vector<double> o;
    o.insert (o.end(), Mv.data(), Mv.data() + Mv.size());
    o.insert (o.end(), Mc.data(), Mc.data() + Mc.size());
    o.insert (o.end(), J.data(), J.data() + J.size());
    bool threw = false;
    try { iface->computeCurrent (MeshLocation::vert); }
    catch (std::logic_error&) { threw = true; }
    o.push_back (threw ? 1.0 : 0.0);
    write_doubles (out, o.data(), o.size());
    return 0;
}

int main (int argc, char** argv)
{
    if (argc != 4) { std::fprintf (stderr, "usage: dropin_driver sod|fail|ct in out\n"); return 2; }
    if (! std::strcmp (argv[1], "sod")) return run_sod (argv[2], argv[3]);
    if (! std::strcmp (argv[1], "fail")) return run_fail (argv[2], argv[3]);
    if (! std::strcmp (argv[1], "ct")) return run_ct (argv[2], argv[3]);
    return 2;
}
