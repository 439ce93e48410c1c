/*---------------------------------------------------------------------------*\
  ref_harness.C - drives the reference's own lduMatrix solver code.

  Test infrastructure only (golden-vector generator).  Linked against
  oracle/_ref/libOpenFOAM.so, which build_ref.py compiles from the
  reference sources.  It reads one record file, runs the reference code named
  by its "mode" record and writes the results to a record file:

    geom   polyMesh from (points, faces, owner, neighbour, patches):
           faceAreas, faceCentres, magFaceAreas, cellCentres, cellVolumes
           (primitiveMeshFaceCentresAndAreas.C, primitiveMeshCellCentresAndVols.C)
    ops    single operations on an lduMatrix: Amul, Tmul, residual, sumA,
           normFactor, DIC/DILU reciprocal diagonals and preconditioning,
           GaussSeidel and DIC smoothing, gSum* reductions
    solve  lduMatrix::solver::New(...)->solve(psi, source) for the solver
           dictionary given as text; for GAMG, an agglomeration built by
           pairGAMGAgglomeration::agglomerate from the given face weights is
           registered first (the faceAreaPair weights need an fvMesh; the
           pairing itself is the reference code path), and the level
           hierarchy and coarse matrices are written too.
    plugin the run-time loading path of a solver library: libs.open(library)
           (dlLibraryTable, as controlDict's libs entry does), then
           lduMatrix::solver::New for the dictionary given as text and
           solve(psi, source), with FatalError thrown as an exception; writes
           whether the library loaded, the selected type, the solver
           performance, or the FatalError message.

  Record file: "CFXREC1\n", then records of
    char name[32]; char dtype[8] ("i4"|"f8"|"s"); int64 count; data
\*---------------------------------------------------------------------------*/

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <iostream>
#include <limits>
#include <list>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "Time.H"
#include "polyMesh.H"
#include "polyPatch.H"
#include "FieldField.H"
#include "lduMatrix.H"
#include "lduPrimitiveMesh.H"
#include "lduInterfaceField.H"
#include "lduSchedule.H"
#include "DICPreconditioner.H"
#include "DILUPreconditioner.H"
#include "pairGAMGAgglomeration.H"
#include "PCG.H"
#include "PBiCGStab.H"
#include "IStringStream.H"
#include "SolverPerformance.H"
#include "GAMGSolver.H"
#include "dlLibraryTable.H"
#include "error.H"
#include "harness_io.H"

using namespace Foam;

// The coarse-level matrices are a private member of GAMGSolver; the harness
// reads them (to pin the device-side coarse assembly) through the standard
// explicit-instantiation access rule.
namespace
{
template<class Tag, typename Tag::type M>
struct memberAccess
{
    friend typename Tag::type get(Tag) { return M; }
};
struct GAMGmatrixLevels
{
    typedef PtrList<lduMatrix> GAMGSolver::*type;
    friend type get(GAMGmatrixLevels);
};
template struct memberAccess<GAMGmatrixLevels, &GAMGSolver::matrixLevels_>;
}

namespace
{




// An lduMesh that owns its addressing and can answer db(), which GAMG needs
// to cache its agglomeration (lduMesh::db() is NotImplemented in the base).
class harnessMesh
:
    public lduPrimitiveMesh
{
    const objectRegistry& db_;

public:

    harnessMesh(const objectRegistry& db, label n, labelList& l, labelList& u)
    :
        lduPrimitiveMesh(n, l, u, UPstream::worldComm, false),
        db_(db)
    {}

    virtual const objectRegistry& db() const { return db_; }
};


// Coupled (cyclic) interfaces for the solver path: an lduInterface holding
// a patch's face cells, and an lduInterfaceField whose update is
// cyclicFvPatchField::updateInterfaceMatrix (cyclicFvPatchField.C:150-174)
// for a scalar field (no transform): result[faceCells] -= coeffs*psi[nbr].
// Like the cyclic field it never marks itself updated, so the reference's
// nonBlocking consume loop applies it once per update, in patch order.
class harnessInterface
:
    public lduInterface
{
    labelList faceCells_;

public:

    explicit harnessInterface(const labelList& fc)
    :
        faceCells_(fc)
    {}

    virtual const labelUList& faceCells() const { return faceCells_; }

    virtual tmp<labelField> interfaceInternalField
    (
        const labelUList& internalData
    ) const
    {
        return tmp<labelField>(new labelField(internalData, faceCells_));
    }

    virtual tmp<labelField> internalFieldTransfer
    (
        const Pstream::commsTypes,
        const labelUList& iF
    ) const
    {
        return tmp<labelField>(new labelField(iF, faceCells_));
    }
};


class harnessCyclicField
:
    public lduInterfaceField
{
    labelList nbrCells_;

public:

    harnessCyclicField(const lduInterface& i, const labelList& nbr)
    :
        lduInterfaceField(i),
        nbrCells_(nbr)
    {}

    virtual void updateInterfaceMatrix
    (
        scalarField& result,
        const scalarField& psiInternal,
        const scalarField& coeffs,
        const direction,
        const Pstream::commsTypes
    ) const
    {
        const scalarField pnf(psiInternal, nbrCells_);
        const labelUList& faceCells = interface().faceCells();
        forAll(faceCells, elemI)
        {
            result[faceCells[elemI]] -= coeffs[elemI]*pnf[elemI];
        }
    }
};


// The interfaces given by the records ifSize (faces per patch), ifCell,
// ifNbr, ifBou and ifInt (faces concatenated in patch order), added to the
// mesh; empty lists without them.
struct harnessInterfaces
{
    // owned by the mesh once added (lduPrimitiveMesh::primitiveInterfaces_)
    UPtrList<harnessInterface> patches;
    PtrList<harnessCyclicField> fields;
    lduInterfacePtrsList ilist;
    lduInterfaceFieldPtrsList ifs;
    Field<Field<scalar>> bou, intc;

    harnessInterfaces(const RecMap& in, harnessMesh& mesh)
    :
        patches(0),
        fields(0),
        ilist(0),
        ifs(0),
        bou(0),
        intc(0)
    {
        if (!has(in, "ifSize")) return;
        const labelList sz(getL(in, "ifSize"));
        const labelList fc(getL(in, "ifCell")), nb(getL(in, "ifNbr"));
        const scalarField b(getF(in, "ifBou"));
        const scalarField ic(has(in, "ifInt") ? getF(in, "ifInt") : getF(in, "ifBou"));
        const label np = sz.size();
        patches.setSize(np);
        fields.setSize(np);
        ilist.setSize(np);
        ifs.setSize(np);
        bou.setSize(np);
        intc.setSize(np);
        label o = 0;
        for (label p = 0; p < np; p++)
        {
            labelList f(sz[p]), n(sz[p]);
            scalarField pb(sz[p]), pi(sz[p]);
            for (label k = 0; k < sz[p]; k++)
            {
                f[k] = fc[o + k];
                n[k] = nb[o + k];
                pb[k] = b[o + k];
                pi[k] = ic[o + k];
            }
            patches.set(p, new harnessInterface(f));
            fields.set(p, new harnessCyclicField(patches[p], n));
            ilist.set(p, &patches[p]);
            ifs.set(p, &fields[p]);
            bou[p] = pb;
            intc[p] = pi;
            o += sz[p];
        }
        mesh.addInterfaces(ilist, lduSchedule());
    }
};


// pairGAMGAgglomeration driven by explicit face weights: the faceAreaPair
// weights (faceAreaPairGAMGAgglomeration.C:55-80) computed from the given
// face-area vectors, then the reference pairing (pairGAMGAgglomerate.C).
class harnessAgglomeration
:
    public pairGAMGAgglomeration
{
public:

    harnessAgglomeration
    (
        const lduMesh& mesh,
        const scalarField& weights,
        const dictionary& dict
    )
    :
        pairGAMGAgglomeration(mesh, dict)
    {
        // pairGAMGAgglomeration::forward_ is a process-global static that
        // starts true; one agglomeration per harness process keeps it so.
        agglomerate(mesh, weights);
    }
};


int runGeom(const RecMap& in, Writer& out, Time& runTime)
{
    const scalarField P(getF(in, "points"));
    const labelList F(getL(in, "faces"));
    labelList own(getL(in, "owner"));
    labelList nei(getL(in, "neighbour"));
    const labelList ps(getL(in, "patchStart"));

    pointField points(P.size()/3);
    forAll(points, i) points[i] = point(P[3*i], P[3*i+1], P[3*i+2]);
    faceList faces(F.size()/4);
    forAll(faces, i)
    {
        face f(4);
        for (int q = 0; q < 4; q++) f[q] = F[4*i+q];
        faces[i] = f;
    }

    polyMesh mesh
    (
        IOobject(polyMesh::defaultRegion, runTime.name(), runTime,
                 IOobject::NO_READ, IOobject::NO_WRITE),
        std::move(points), std::move(faces), std::move(own), std::move(nei),
        false
    );

    List<polyPatch*> patches(ps.size() - 1);
    forAll(patches, p)
    {
        patches[p] = new polyPatch
        (
            "patch" + Foam::name(p), ps[p+1] - ps[p], ps[p], p, mesh.boundary()
        );
    }
    mesh.addPatches(patches, false);

    out.vec("Sf", mesh.faceAreas());
    out.vec("Cf", mesh.faceCentres());
    out.f8("magSf", mesh.magFaceAreas());
    out.vec("C", mesh.cellCentres());
    out.f8("V", mesh.cellVolumes());
    return 0;
}


void buildMatrix(lduMatrix& A, const RecMap& in, label nCells, label nFaces)
{
    A.diag(nCells) = getF(in, "diag");
    A.upper(nFaces) = getF(in, "upper");
    if (has(in, "lower")) A.lower(nFaces) = getF(in, "lower");
}


int runOps(const RecMap& in, Writer& out, Time& runTime)
{
    labelList l(getL(in, "l")), u(getL(in, "u"));
    const scalarField x(getF(in, "x")), b(getF(in, "b"));
    const label nCells = x.size(), nFaces = l.size();
    harnessMesh mesh(runTime, nCells, l, u);
    harnessInterfaces hi(in, mesh);
    lduMatrix A(mesh);
    buildMatrix(A, in, nCells, nFaces);

    Field<Field<scalar>>& bou = hi.bou;
    Field<Field<scalar>>& intc = hi.intc;
    lduInterfaceFieldPtrsList& ifs = hi.ifs;

    scalarField y(nCells);
    A.Amul(y, x, bou, ifs, 0);
    out.f8("Amul", y);
    A.Tmul(y, x, intc, ifs, 0);
    out.f8("Tmul", y);
    A.residual(y, x, b, bou, ifs, 0);
    out.f8("residual", y);
    A.sumA(y, bou, ifs);
    out.f8("sumA", y);

    out.f8("sumMag", gSumMag(b));
    out.f8("sumProd", gSumProd(x, b));
    out.f8("sumSqr", gSumSqr(b));
    out.f8("sum", gSum(b));
    out.f8("average", gAverage(x));

    // normFactor via a throw-away solver object (the base implementation)
    {
        IStringStream is
        (
            A.symmetric()
          ? "{ solver PCG; preconditioner none; }"
          : "{ solver PBiCGStab; preconditioner none; }"
        );
        dictionary d(is);
        autoPtr<lduMatrix::solver> s =
            lduMatrix::solver::New("x", A, bou, intc, ifs, d);
        scalarField Ax(nCells), tmp(nCells);
        A.Amul(Ax, x, bou, ifs, 0);
        out.f8("normFactor", s->normFactor(x, b, Ax, tmp));
    }

    if (A.symmetric())
    {
        scalarField rD(A.diag());
        DICPreconditioner::calcReciprocalD(rD, A);
        out.f8("DIC_rD", rD);
        IStringStream is("{ solver PCG; preconditioner DIC; }");
        dictionary d(is);
        autoPtr<lduMatrix::solver> s =
            lduMatrix::solver::New("x", A, bou, intc, ifs, d);
        autoPtr<lduMatrix::preconditioner> p =
            lduMatrix::preconditioner::New(s(), d);
        p->precondition(y, b, 0);
        out.f8("DIC_precondition", y);

        IStringStream is2("{ smoother DIC; }");
        dictionary d2(is2);
        autoPtr<lduMatrix::smoother> sm =
            lduMatrix::smoother::New("x", A, bou, intc, ifs, d2);
        scalarField psi(x);
        sm->smooth(psi, b, 0, 2);
        out.f8("DIC_smooth2", psi);
    }
    else
    {
        scalarField rD(A.diag());
        DILUPreconditioner::calcReciprocalD(rD, A);
        out.f8("DILU_rD", rD);
        IStringStream is("{ solver PBiCGStab; preconditioner DILU; }");
        dictionary d(is);
        autoPtr<lduMatrix::solver> s =
            lduMatrix::solver::New("x", A, bou, intc, ifs, d);
        autoPtr<lduMatrix::preconditioner> p =
            lduMatrix::preconditioner::New(s(), d);
        p->precondition(y, b, 0);
        out.f8("DILU_precondition", y);
        p->preconditionT(y, b, 0);
        out.f8("DILU_preconditionT", y);
    }

    {
        IStringStream is("{ smoother GaussSeidel; }");
        dictionary d(is);
        autoPtr<lduMatrix::smoother> sm =
            lduMatrix::smoother::New("x", A, bou, intc, ifs, d);
        scalarField psi(x);
        sm->smooth(psi, b, 0, 1);
        out.f8("GS_smooth1", psi);
        sm->smooth(psi, b, 0, 2);
        out.f8("GS_smooth3", psi);
    }

    // the other smoothers of the run-time table, 2 sweeps from x
    {
        std::vector<std::string> names;
        names.push_back("symGaussSeidel");
        if (A.symmetric())
        {
            names.push_back("DICGaussSeidel");
        }
        else
        {
            names.push_back("DILU");
            names.push_back("DILUGaussSeidel");
        }
        for (const std::string& nm : names)
        {
            IStringStream is("{ smoother " + nm + "; }");
            dictionary d(is);
            autoPtr<lduMatrix::smoother> sm =
                lduMatrix::smoother::New("x", A, bou, intc, ifs, d);
            scalarField psi(x);
            sm->smooth(psi, b, 0, 2);
            out.f8(nm + "_smooth2", psi);
        }
    }

    out.i4("ownerStart", mesh.lduAddr().ownerStartAddr());
    out.i4("losort", mesh.lduAddr().losortAddr());
    out.i4("losortStart", mesh.lduAddr().losortStartAddr());
    return 0;
}


int runSolve(const RecMap& in, Writer& out, Time& runTime)
{
    labelList l(getL(in, "l")), u(getL(in, "u"));
    const scalarField source(getF(in, "source"));
    scalarField psi(getF(in, "psi"));
    const label nCells = source.size(), nFaces = l.size();
    harnessMesh mesh(runTime, nCells, l, u);
    harnessInterfaces hi(in, mesh);
    lduMatrix A(mesh);
    buildMatrix(A, in, nCells, nFaces);

    IStringStream is(getS(in, "dict"));
    dictionary dict(is);

    Field<Field<scalar>>& bou = hi.bou;
    Field<Field<scalar>>& intc = hi.intc;
    lduInterfaceFieldPtrsList& ifs = hi.ifs;

    const word solverName(dict.lookup("solver"));
    // GAMG, or a solver preconditioned by GAMG (a preconditioner
    // dictionary with preconditioner GAMG and the GAMG keys): the
    // agglomeration from the given weights
    const bool gamgPre =
        dict.isDict("preconditioner")
     && word(dict.subDict("preconditioner").lookup("preconditioner")) == "GAMG";
    if (solverName == "GAMG" || gamgPre)
    {
        const scalarField w(getF(in, "weights"));
        harnessAgglomeration* agg = new harnessAgglomeration
        (
            mesh, w, gamgPre ? dict.subDict("preconditioner") : dict
        );
        regIOobject::store(static_cast<GAMGAgglomeration*>(agg));
    }

    autoPtr<lduMatrix::solver> s =
        lduMatrix::solver::New("psi", A, bou, intc, ifs, dict);
    solverPerformance perf = s->solve(psi, source, 0);

    out.f8("psi", psi);
    out.f8("initialResidual", perf.initialResidual());
    out.f8("finalResidual", perf.finalResidual());
    out.i4("nIterations", perf.nIterations());
    out.i4("converged", perf.converged() ? 1 : 0);
    out.i4("singular", perf.singular() ? 1 : 0);
    out.put("solverName", "s", perf.solverName().c_str(), perf.solverName().size(), 1);

    if (solverName == "GAMG")
    {
        const GAMGSolver& g = refCast<const GAMGSolver>(s());
        const GAMGAgglomeration& agg =
            mesh.db().lookupObject<GAMGAgglomeration>(GAMGAgglomeration::typeName);
        out.i4("nLevels", agg.size());
        for (label i = 0; i < agg.size(); i++)
        {
            const std::string k = std::to_string(i);
            out.i4("restrict" + k, agg.restrictAddressing(i));
            out.i4("faceRestrict" + k, agg.faceRestrictAddressing(i));
            const boolList& fl = agg.faceFlipMap(i);
            labelList fli(fl.size());
            forAll(fl, j) fli[j] = fl[j] ? 1 : 0;
            out.i4("faceFlip" + k, fli);
            out.i4("nCells" + k, agg.nCells(i));
            out.i4("nFaces" + k, agg.nFaces(i));
            const lduAddressing& ca = agg.meshLevel(i + 1).lduAddr();
            out.i4("coarseL" + k, ca.lowerAddr());
            out.i4("coarseU" + k, ca.upperAddr());
            const lduMatrix& cm = (g.*get(GAMGmatrixLevels()))[i];
            out.f8("coarseDiag" + k, cm.diag());
            out.f8("coarseUpper" + k, cm.upper());
            if (cm.hasLower()) out.f8("coarseLower" + k, cm.lower());
        }
    }
    return 0;
}

int runPlugin(const RecMap& in, Writer& out, Time& runTime)
{
    labelList l(getL(in, "l")), u(getL(in, "u"));
    const scalarField source(getF(in, "source"));
    scalarField psi(getF(in, "psi"));
    const label nCells = source.size(), nFaces = l.size();
    harnessMesh mesh(runTime, nCells, l, u);
    harnessInterfaces hi(in, mesh);
    lduMatrix A(mesh);
    buildMatrix(A, in, nCells, nFaces);

    const std::string lib = getS(in, "library");
    const bool loaded = lib.empty() ? false : libs.open(fileName(lib));
    out.i4("loaded", loaded ? 1 : 0);

    FatalError.throwExceptions();
    FatalIOError.throwExceptions();
    try
    {
        IStringStream is(getS(in, "dict"));
        dictionary dict(is);
        autoPtr<lduMatrix::solver> s =
            lduMatrix::solver::New("psi", A, hi.bou, hi.intc, hi.ifs, dict);
        const std::string type(s->type());
        out.put("type", "s", type.c_str(), type.size(), 1);
        solverPerformance perf = s->solve(psi, source, 0);
        out.f8("psi", psi);
        out.f8("finalResidual", perf.finalResidual());
        out.i4("nIterations", perf.nIterations());
        out.put("solverName", "s", perf.solverName().c_str(), perf.solverName().size(), 1);
    }
    catch (const Foam::error& e)
    {
        const std::string msg(e.message());
        out.put("fatal", "s", msg.c_str(), msg.size(), 1);
    }
    return 0;
}

} // namespace


int main(int argc, char* argv[])
{
    if (argc != 3)
    {
        std::fprintf(stderr, "usage: ref_harness in.rec out.rec\n");
        return 2;
    }
    const RecMap in = readRecs(argv[1]);
    const std::string mode = getS(in, "mode");

    const char* tmp = std::getenv("CFX_HARNESS_ROOT");
    const fileName root(tmp ? tmp : "/tmp");
    Time runTime(root, "cfxcase", false);

    Writer out(argv[2]);
    if (mode == "geom") return runGeom(in, out, runTime);
    if (mode == "ops") return runOps(in, out, runTime);
    if (mode == "solve") return runSolve(in, out, runTime);
    if (mode == "plugin") return runPlugin(in, out, runTime);
    std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
    return 2;
}
