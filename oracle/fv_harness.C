/*---------------------------------------------------------------------------*\
  fv_harness.C - drives the reference's own finite-volume assembly.

  Test infrastructure only (golden-vector generator).  Linked against
  oracle/_ref/libfiniteVolume.so and libOpenFOAM.so, which build_ref_fv.py and
  build_ref.py compile from the reference sources.  It reads one record file
  (harness_io.H) describing a hex mesh (points, faces, owner, neighbour,
  patchStart), psi's boundary condition per patch (patchBC: 0 zeroGradient,
  1 fixedValue, 2 fixedGradient, with bcValue per boundary face: the value
  or the gradient; 3 cyclic, patches 2i and 2i+1 coupled face by face), the
  fields and the terms, builds an fvMesh and
  volScalarField T in the case directory (whose system/fvSchemes selects
  Euler, Gauss upwind or linear, Gauss linear uncorrected), assembles

      fvm::ddt(T) + fvm::div(phi, T) +/- fvm::laplacian(gamma, T) == su

  with each term optional, as a solver application writes it, and writes the
  lduMatrix and source that fvMatrix::solveSegregated hands to the linear
  solver (diag with addBoundaryDiag, source with addBoundarySource without
  the coupled patches), the cyclic patches' interfaces (face cells, the
  partner's face cells, boundaryCoeffs and internalCoeffs, which the solver
  receives as interfaceBouCoeffs and interfaceIntCoeffs), and the
  geometry the schemes used (magSf, nonOrthDeltaCoeffs, weights, V, the
  patches' magSf and deltaCoeffs).  With a "dict" record it then solves the
  equation as a solver application does, fvMatrix::solve(dict) (segregated:
  addBoundaryDiag/Source, lduMatrix::solver::New on the fvMesh, so GAMG
  agglomerates with faceAreaPair from the mesh's own Sf), starting from psi0
  (or zero), and writes psi, the solver performance and, for GAMG, the
  agglomeration levels.
\*---------------------------------------------------------------------------*/

#include "Time.H"
#include "fvMesh.H"
#include "polyPatch.H"
#include "volFields.H"
#include "surfaceFields.H"
#include "fvMatrices.H"
#include "fvmDdt.H"
#include "fvmDiv.H"
#include "fvmLaplacian.H"
#include "fixedValueFvPatchFields.H"
#include "zeroGradientFvPatchFields.H"
#include "fixedGradientFvPatchFields.H"
#include "cyclicPolyPatch.H"
#include "cyclicFvPatchFields.H"
#include "GAMGAgglomeration.H"
#include "IStringStream.H"
#include "harness_io.H"

using namespace Foam;

// fvMatrix::addBoundaryDiag / addBoundarySource are protected; the harness
// calls the reference's own functions through the explicit-instantiation
// access rule.
namespace
{
template<class Tag, typename Tag::type M>
struct memberAccess
{
    friend typename Tag::type get(Tag) { return M; }
};
struct fvmAddBoundaryDiag
{
    typedef void (fvScalarMatrix::*type)(scalarField&, const direction) const;
    friend type get(fvmAddBoundaryDiag);
};
struct fvmAddBoundarySource
{
    typedef void (fvScalarMatrix::*type)(scalarField&, const bool) const;
    friend type get(fvmAddBoundarySource);
};
template struct memberAccess<fvmAddBoundaryDiag, &fvScalarMatrix::addBoundaryDiag>;
template struct memberAccess<fvmAddBoundarySource, &fvScalarMatrix::addBoundarySource>;


// A field of the boundary faces (patch order), one slice per patch
template<class F>
void setBoundary(F& bf, const labelList& ps, label nI, const scalarField& all)
{
    forAll(bf, p)
    {
        const label n = ps[p + 1] - ps[p];
        scalarField v(n);
        for (label k = 0; k < n; k++) v[k] = all[ps[p] - nI + k];
        bf[p] = v;
    }
}


int runFvm(const RecMap& in, Writer& out, Time& runTime)
{
    const scalarField P(getF(in, "points"));
    const labelList F(getL(in, "faces"));
    labelList own(getL(in, "owner"));
    labelList nei(getL(in, "neighbour"));
    const labelList ps(getL(in, "patchStart"));
    const labelList patchBC(getL(in, "patchBC"));

    pointField points(P.size()/3);
    forAll(points, i) points[i] = point(P[3*i], P[3*i+1], P[3*i+2]);
    faceList faces(F.size()/4);
    forAll(faces, i)
    {
        face f(4);
        for (int q = 0; q < 4; q++) f[q] = F[4*i+q];
        faces[i] = f;
    }

    fvMesh mesh
    (
        IOobject(fvMesh::defaultRegion, runTime.name(), runTime,
                 IOobject::NO_READ, IOobject::NO_WRITE),
        std::move(points), std::move(faces), std::move(own), std::move(nei),
        false
    );
    List<polyPatch*> patches(ps.size() - 1);
    forAll(patches, p)
    {
        if (patchBC[p] == 3)
        {
            patches[p] = new cyclicPolyPatch
            (
                "patch" + Foam::name(p), ps[p+1] - ps[p], ps[p], p,
                static_cast<const polyMesh&>(mesh).boundary(),
                "patch" + Foam::name(p % 2 ? p - 1 : p + 1)
            );
        }
        else
        {
            patches[p] = new polyPatch
            (
                "patch" + Foam::name(p), ps[p+1] - ps[p], ps[p], p,
                static_cast<const polyMesh&>(mesh).boundary()
            );
        }
    }
    mesh.addFvPatches(patches, true);
    const label nI = mesh.nInternalFaces();

    // psi with its boundary conditions and old-time value (fixedGradient
    // has no null constructor in the run-time table: those patches are
    // replaced after construction)
    wordList types(patches.size());
    forAll(types, p)
    {
        types[p] =
            patchBC[p] == 1 ? fixedValueFvPatchScalarField::typeName
          : patchBC[p] == 3 ? cyclicFvPatchScalarField::typeName
          : zeroGradientFvPatchScalarField::typeName;
    }
    volScalarField T
    (
        IOobject("T", runTime.name(), mesh, IOobject::NO_READ, IOobject::NO_WRITE),
        mesh,
        dimensionedScalar(dimless, 0),
        types
    );
    if (has(in, "psi0")) T.primitiveFieldRef() = getF(in, "psi0");
    const scalarField bcValue(getF(in, "bcValue"));
    forAll(types, p)
    {
        const label n = ps[p + 1] - ps[p];
        scalarField v(n);
        for (label k = 0; k < n; k++) v[k] = bcValue[ps[p] - nI + k];
        if (patchBC[p] == 1)
        {
            T.boundaryFieldRef()[p] == v;
        }
        else if (patchBC[p] == 2)
        {
            fixedGradientFvPatchScalarField* fg =
                new fixedGradientFvPatchScalarField(mesh.boundary()[p], T);
            fg->gradient() = v;
            T.boundaryFieldRef().set(p, fg);
            T.boundaryFieldRef()[p].evaluate();
        }
    }
    T.oldTime();

    surfaceScalarField phi
    (
        IOobject("phi", runTime.name(), mesh, IOobject::NO_READ, IOobject::NO_WRITE),
        mesh,
        dimensionedScalar(dimVolume/dimTime, 0)
    );
    const bool div = has(in, "phi");
    if (div)
    {
        phi.primitiveFieldRef() = getF(in, "phi");
        setBoundary(phi.boundaryFieldRef(), ps, nI, getF(in, "phiB"));
    }
    surfaceScalarField gammaf
    (
        IOobject("gammaf", runTime.name(), mesh, IOobject::NO_READ, IOobject::NO_WRITE),
        mesh,
        dimensionedScalar(dimArea/dimTime, 0)
    );
    const bool faceGamma = has(in, "gamma");
    if (faceGamma)
    {
        gammaf.primitiveFieldRef() = getF(in, "gamma");
        setBoundary(gammaf.boundaryFieldRef(), ps, nI, getF(in, "gammaB"));
    }
    const dimensionedScalar gammaU
    (
        "DT", dimArea/dimTime,
        has(in, "gammaUniform") ? getF(in, "gammaUniform")[0] : 1.0
    );
    volScalarField::Internal su
    (
        IOobject("su", runTime.name(), mesh, IOobject::NO_READ, IOobject::NO_WRITE),
        mesh,
        dimensionedScalar(dimless/dimTime, 0)
    );
    if (has(in, "su")) su.primitiveFieldRef() = getF(in, "su");

    // the equation, term by term as a solver writes it
    const bool ddt = has(in, "deltaT");
    const label lapSign = has(in, "lapSign") ? getL(in, "lapSign")[0] : 0;
    auto lap = [&]()
    {
        return faceGamma ? fvm::laplacian(gammaf, T) : fvm::laplacian(gammaU, T);
    };
    autoPtr<fvScalarMatrix> E;
    if (ddt) E.set(new fvScalarMatrix(fvm::ddt(T)));
    if (div)
    {
        if (E.valid()) E() += fvm::div(phi, T);
        else E.set(new fvScalarMatrix(fvm::div(phi, T)));
    }
    if (lapSign)
    {
        if (E.valid())
        {
            if (lapSign > 0) E() += lap();
            else E() -= lap();
        }
        else
        {
            E.set(new fvScalarMatrix(lapSign > 0 ? lap() : -lap()));
        }
    }
    if (!E.valid())
    {
        std::fprintf(stderr, "no term\n");
        return 2;
    }
    tmp<fvScalarMatrix> tM =
        has(in, "su") ? (E() == su) : tmp<fvScalarMatrix>(new fvScalarMatrix(E()));
    const fvScalarMatrix& M = tM();

    // what fvMatrix::solveSegregated hands to the solver
    scalarField diag(M.diag());
    (M.*get(fvmAddBoundaryDiag()))(diag, 0);
    scalarField source(M.source());
    (M.*get(fvmAddBoundarySource()))(source, false);
    out.f8("diag", diag);
    out.f8("upper", M.upper());
    if (M.hasLower()) out.f8("lower", M.lower());
    out.f8("source", source);
    {
        fvScalarMatrix& Mw = tM.ref();  // the coefficient accessors are non-const
        DynamicList<label> ifSize, ifCell, ifNbr;
        DynamicList<scalar> ifBou, ifInt;
        forAll(mesh.boundary(), p)
        {
            if (patchBC[p] != 3) continue;
            const labelUList& fc = mesh.boundary()[p].faceCells();
            const labelUList& nc =
                mesh.boundary()[p % 2 ? p - 1 : p + 1].faceCells();
            ifSize.append(fc.size());
            forAll(fc, k)
            {
                ifCell.append(fc[k]);
                ifNbr.append(nc[k]);
                ifBou.append(Mw.boundaryCoeffs()[p][k]);
                ifInt.append(Mw.internalCoeffs()[p][k]);
            }
        }
        if (ifSize.size())
        {
            out.i4("ifSize", labelList(ifSize));
            out.i4("ifCell", labelList(ifCell));
            out.i4("ifNbr", labelList(ifNbr));
            out.f8("ifBou", scalarField(ifBou));
            out.f8("ifInt", scalarField(ifInt));
        }
    }

    // the geometry the schemes used
    out.f8("magSf", mesh.magSf().primitiveField());
    out.f8("deltaCoeffs", mesh.nonOrthDeltaCoeffs().primitiveField());
    out.f8("weights", mesh.weights().primitiveField());
    scalarField Vc(mesh.nCells());
    forAll(Vc, c) Vc[c] = mesh.V()[c];
    out.f8("V", Vc);
    DynamicList<label> bCell;
    DynamicList<scalar> magSfB, deltaCoeffsB;
    forAll(mesh.boundary(), p)
    {
        const fvPatch& fp = mesh.boundary()[p];
        const labelUList& fc = fp.faceCells();
        // the Laplacian takes a coupled patch's coefficients from the snGrad
        // scheme's deltaCoeffs (nonOrthDeltaCoeffs), an uncoupled patch's
        // from the patch's own deltaCoeffs (gaussLaplacianScheme.C:64-86)
        const scalarField dc
        (
            fp.coupled()
          ? scalarField(mesh.nonOrthDeltaCoeffs().boundaryField()[p])
          : scalarField(fp.deltaCoeffs())
        );
        forAll(fc, k)
        {
            bCell.append(fc[k]);
            magSfB.append(fp.magSf()[k]);
            deltaCoeffsB.append(dc[k]);
        }
    }
    out.i4("bCell", labelList(bCell));
    out.f8("magSfB", scalarField(magSfB));
    out.f8("deltaCoeffsB", scalarField(deltaCoeffsB));

    if (has(in, "dict"))
    {
        IStringStream is(getS(in, "dict"));
        const dictionary dict(is);
        if (!has(in, "psi0")) T.primitiveFieldRef() = 0;
        const solverPerformance perf = tM.ref().solve(dict);
        out.f8("psi", T.primitiveField());
        out.f8("initialResidual", perf.initialResidual());
        out.f8("finalResidual", perf.finalResidual());
        out.i4("nIterations", perf.nIterations());
        out.i4("converged", perf.converged() ? 1 : 0);
        out.put("solverName", "s", perf.solverName().c_str(), perf.solverName().size(), 1);
        const objectRegistry& db = static_cast<const lduMesh&>(mesh).db();
        if (db.foundObject<GAMGAgglomeration>(GAMGAgglomeration::typeName))
        {
            const GAMGAgglomeration& agg =
                db.lookupObject<GAMGAgglomeration>(GAMGAgglomeration::typeName);
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
            }
        }
    }
    return 0;
}

} // End anonymous namespace


int main(int argc, char* argv[])
{
    if (argc != 3)
    {
        std::fprintf(stderr, "usage: fv_harness in.rec out.rec\n");
        return 2;
    }
    const RecMap in = readRecs(argv[1]);
    const char* tmp = std::getenv("CFX_HARNESS_ROOT");
    const fileName root(tmp ? tmp : "/tmp");
    Time runTime(root, "cfxcase", false);
    if (has(in, "deltaT")) runTime.setDeltaT(getF(in, "deltaT")[0]);
    Writer out(argv[2]);
    return runFvm(in, out, runTime);
}
