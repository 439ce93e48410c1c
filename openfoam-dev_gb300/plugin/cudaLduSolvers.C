/*---------------------------------------------------------------------------*\
  cudaLduSolvers.C - OpenFOAM run-time selectable solvers cudaPCG,
  cudaPBiCGStab, cudaGAMG and cudaSmoothSolver backed by
  libcudaLduSolvers.so (include/cfx.h).

  Build into libcudaLduSolvers_OpenFOAM.so with wmake (Make/files: this file;
  Make/options: -I<repo>/include, -L<repo>/openfoam-dev_gb300/lib
  -lcudaLduSolvers) and load it from system/controlDict:

      libs ("libcudaLduSolvers_OpenFOAM.so");

  then select it in system/fvSolution, e.g.

      p { solver cudaGAMG; smoother GaussSeidel; nPreSweeps 2;
          tolerance 1e-8; relTol 0; precision mixed; }

  Registration follows the reference's solvers (PCG.C:30-36,
  PBiCGStab.C:30-39, GAMGSolver.C:34-43, smoothSolver.C:32-38): cudaPCG in
  the symmetric table, cudaPBiCGStab, cudaGAMG and cudaSmoothSolver in both.  The solver object is constructed per
  fvMatrix::solve (fvScalarMatrix.C:162-170); the device copies of the
  addressing, level schedules and GAMG hierarchy live in a process-wide
  cache keyed by the lduMesh, and the coefficients are re-uploaded on every
  solve.  Cyclic coupled interfaces are passed through (each patch's face
  cells, its partner's face cells, interfaceBouCoeffs and
  interfaceIntCoeffs); the library builds GAMG's coarse cyclic interfaces
  itself.  Any other coupled interface (processor) is refused with
  FatalError.
\*---------------------------------------------------------------------------*/

#include "lduMatrix.H"
#include "GAMGAgglomeration.H"
#include "cyclicLduInterface.H"
#include "addToRunTimeSelectionTable.H"

#include "cfx.h"

#include <map>

namespace Foam
{

class cudaLduSolver
:
    public lduMatrix::solver
{
protected:

    struct Entry
    {
        cfx_mesh* mesh = nullptr;
        cfx_matrix* mat = nullptr;
        label nCells = -1;
        label nFaces = -1;
        bool sym = true;
        bool gamg = false;
        bool interfaces = false;  // the mesh's cyclic interfaces are set
    };

    static cfx_ctx* context()
    {
        static cfx_ctx* ctx = nullptr;
        if (!ctx && cfx_ctx_create(0, &ctx) != CFX_OK)
        {
            FatalErrorInFunction
                << "cudaLduSolvers: " << cfx_last_error() << exit(FatalError);
        }
        return ctx;
    }

    static std::map<const lduMesh*, Entry>& cache()
    {
        static std::map<const lduMesh*, Entry> c;
        return c;
    }

    static void check(int status, const char* what)
    {
        if (status != CFX_OK)
        {
            FatalErrorInFunction
                << what << ": " << cfx_last_error() << exit(FatalError);
        }
    }

    //- The device matrix for this solve: addressing cached per mesh,
    //  coefficients uploaded now
    Entry& deviceMatrix() const
    {
        // coupled interfaces: cyclic ones (faceCells, the neighbour patch's
        // faceCells, in interface order); processor interfaces are not
        // supported on one GPU
        DynamicList<label> ifSize, ifCells, ifNbr, ifPartner;
        DynamicList<scalar> ifBou, ifInt;
        // the library numbers the set interfaces only
        labelList libIndex(interfaces_.size(), -1);
        {
            label k = 0;
            forAll(interfaces_, patchi)
            {
                if (interfaces_.set(patchi)) libIndex[patchi] = k++;
            }
        }
        forAll(interfaces_, patchi)
        {
            if (!interfaces_.set(patchi)) continue;
            const lduInterface& li = interfaces_[patchi].interface();
            if (!isA<cyclicLduInterface>(li))
            {
                FatalErrorInFunction
                    << "cudaLduSolvers: only cyclic coupled interfaces are "
                    << "supported (patch " << patchi << ")"
                    << exit(FatalError);
            }
            const label nbrI =
                refCast<const cyclicLduInterface>(li).nbrPatchIndex();
            const labelUList& fc = li.faceCells();
            const labelUList& nc = interfaces_[nbrI].interface().faceCells();
            ifSize.append(fc.size());
            ifPartner.append(libIndex[nbrI]);
            forAll(fc, i)
            {
                ifCells.append(fc[i]);
                ifNbr.append(nc[i]);
                ifBou.append(interfaceBouCoeffs_[patchi][i]);
                ifInt.append(interfaceIntCoeffs_[patchi][i]);
            }
        }

        const lduAddressing& addr = matrix_.lduAddr();
        Entry& e = cache()[&matrix_.mesh()];
        const label nCells = addr.size();
        const label nFaces = addr.lowerAddr().size();
        const bool sym = matrix_.symmetric();

        if (e.mesh && (e.nCells != nCells || e.nFaces != nFaces))
        {
            cfx_matrix_destroy(e.mat);
            cfx_mesh_destroy(e.mesh);
            e = Entry();
        }
        if (!e.mesh)
        {
            check
            (
                cfx_mesh_create
                (
                    context(), nCells, nFaces,
                    addr.lowerAddr().cdata(), addr.upperAddr().cdata(),
                    &e.mesh
                ),
                "cfx_mesh_create"
            );
            e.nCells = nCells;
            e.nFaces = nFaces;
        }
        if (ifSize.size() && !e.interfaces)
        {
            check
            (
                cfx_mesh_set_interfaces
                (
                    e.mesh, ifSize.size(), ifSize.cdata(), ifCells.cdata(),
                    ifNbr.cdata()
                ),
                "cfx_mesh_set_interfaces"
            );
            // the direct coarsest-level solve reads the partner patches'
            // coefficients (LUscalarMatrix::convert)
            check
            (
                cfx_mesh_set_interface_partners(e.mesh, ifPartner.cdata()),
                "cfx_mesh_set_interface_partners"
            );
            e.interfaces = true;
        }

        const scalar* lower = sym ? nullptr : matrix_.lower().cdata();
        if (!e.mat || e.sym != sym)
        {
            if (e.mat) cfx_matrix_destroy(e.mat);
            check
            (
                cfx_matrix_create
                (
                    e.mesh, matrix_.diag().cdata(), matrix_.upper().cdata(),
                    lower, &e.mat
                ),
                "cfx_matrix_create"
            );
            e.sym = sym;
        }
        else
        {
            check
            (
                cfx_matrix_update
                (
                    e.mat, matrix_.diag().cdata(), matrix_.upper().cdata(), lower
                ),
                "cfx_matrix_update"
            );
        }
        if (ifSize.size())
        {
            check
            (
                cfx_matrix_set_interface_coeffs
                (
                    e.mat, ifBou.cdata(), ifInt.cdata()
                ),
                "cfx_matrix_set_interface_coeffs"
            );
        }
        return e;
    }

    //- The preconditioner's dictionary when it is given as one (the
    //  "preconditioner { preconditioner GAMG; ... }" form read by
    //  lduMatrix::preconditioner::getName, lduMatrixPreconditioner.C:38-58)
    const dictionary* preconditionerDict() const
    {
        return controlDict_.isDict("preconditioner")
            ? &controlDict_.subDict("preconditioner")
            : nullptr;
    }

    //- The GAMG hierarchy of the entry from the reference's own
    //  agglomeration (faceAreaPair on an fvMesh), cached in the mesh
    //  registry (GAMGAgglomeration.C:349-400); its restriction maps define
    //  the device levels.
    void gamgLevels(Entry& e, const dictionary& gamgDict) const
    {
        if (e.gamg) return;
        const GAMGAgglomeration& agg =
            GAMGAgglomeration::New(matrix_, gamgDict);
        const label nLevels = agg.size();
        List<const label*> maps(nLevels);
        labelList nCoarse(nLevels);
        for (label i = 0; i < nLevels; i++)
        {
            maps[i] = agg.restrictAddressing(i).cdata();
            nCoarse[i] = agg.nCells(i);
        }
        check
        (
            cfx_gamg_set_levels(e.mesh, nLevels, maps.cdata(), nCoarse.cdata()),
            "cfx_gamg_set_levels"
        );
        e.gamg = true;
    }

    //- The preconditioner's name as lduMatrix::preconditioner::New reads
    //  it (lduMatrixPreconditioner.C:60-75; the keyword is required), checked
    //  against the reference's own run-time tables with its error text
    //  (lduMatrixPreconditioner.C:96-136), then against what the device
    //  implements
    word preconditionerName() const
    {
        const entry& pe =
            controlDict_.lookupEntry("preconditioner", false, false);
        word name;
        if (pe.isDict())
        {
            pe.dict().lookup("preconditioner") >> name;
        }
        else
        {
            pe.stream() >> name;
        }
        const dictionary& pc = pe.isDict() ? pe.dict() : dictionary::null;
        if (matrix_.diagonal()) return name;
        if (matrix_.symmetric())
        {
            if (!lduMatrix::preconditioner::symMatrixConstructorTablePtr_->found(name))
            {
                FatalIOErrorInFunction(pc)
                    << "Unknown symmetric matrix preconditioner "
                    << name << nl << nl
                    << "Valid symmetric matrix preconditioners :" << endl
                    << lduMatrix::preconditioner::symMatrixConstructorTablePtr_->sortedToc()
                    << exit(FatalIOError);
            }
        }
        else if
        (
            !lduMatrix::preconditioner::asymMatrixConstructorTablePtr_->found(name)
        )
        {
            FatalIOErrorInFunction(pc)
                << "Unknown asymmetric matrix preconditioner "
                << name << nl << nl
                << "Valid asymmetric matrix preconditioners :" << endl
                << lduMatrix::preconditioner::asymMatrixConstructorTablePtr_->sortedToc()
                << exit(FatalIOError);
        }
        static const wordList onDevice
        ({"none", "diagonal", "DIC", "FDIC", "DILU", "GAMG"});
        if (findIndex(onDevice, name) < 0)
        {
            FatalIOErrorInFunction(controlDict_)
                << "cudaLduSolvers: preconditioner " << name
                << " is not available on the GPU; available: " << onDevice
                << exit(FatalIOError);
        }
        return name;
    }

    //- The smoother's name as lduMatrix::smoother::New reads it
    //  (lduMatrixSmoother.C:40-60, the keyword required), checked against
    //  the reference's run-time tables with its error text
    //  (lduMatrixSmoother.C:102-147), then against what the device implements
    word smootherName(const dictionary& d) const
    {
        const entry& se = d.lookupEntry("smoother", false, false);
        word name;
        if (se.isDict())
        {
            se.dict().lookup("smoother") >> name;
        }
        else
        {
            se.stream() >> name;
        }
        if (matrix_.diagonal()) return name;
        if (matrix_.symmetric())
        {
            if (!lduMatrix::smoother::symMatrixConstructorTablePtr_->found(name))
            {
                FatalIOErrorInFunction(d)
                    << "Unknown symmetric matrix smoother "
                    << name << nl << nl
                    << "Valid symmetric matrix smoothers are :" << endl
                    << lduMatrix::smoother::symMatrixConstructorTablePtr_->sortedToc()
                    << exit(FatalIOError);
            }
        }
        else if
        (
            !lduMatrix::smoother::asymMatrixConstructorTablePtr_->found(name)
        )
        {
            FatalIOErrorInFunction(d)
                << "Unknown asymmetric matrix smoother "
                << name << nl << nl
                << "Valid asymmetric matrix smoothers are :" << endl
                << lduMatrix::smoother::asymMatrixConstructorTablePtr_->sortedToc()
                << exit(FatalIOError);
        }
        static const wordList onDevice
        ({
            "GaussSeidel", "symGaussSeidel", "nonBlockingGaussSeidel", "DIC",
            "FDIC", "DILU", "DICGaussSeidel", "DILUGaussSeidel"
        });
        if (findIndex(onDevice, name) < 0)
        {
            FatalIOErrorInFunction(d)
                << "cudaLduSolvers: smoother " << name
                << " is not available on the GPU; available: " << onDevice
                << exit(FatalIOError);
        }
        return name;
    }

    //- The solver controls, read and checked before any device work
    cfx_controls controls(int solverType) const
    {
        cfx_controls c;
        cfx_default_controls(&c);
        c.solver = solverType;
        c.tolerance = tolerance_;
        c.relTol = relTol_;
        c.maxIter = maxIter_;
        c.minIter = minIter_;
        const dictionary* pd = preconditionerDict();
        // Krylov solvers construct a preconditioner (PCG.C:104-112,
        // PBiCGStab.C:104-112, PBiCG.C:104-112); GAMG and smoothSolver do not
        const bool krylov =
            solverType == CFX_SOLVER_PCG || solverType == CFX_SOLVER_PBICGSTAB
         || solverType == CFX_SOLVER_PBICG;
        const word pre(krylov ? preconditionerName() : word("none"));
        c.preconditioner =
            pre == "DIC" ? CFX_PRE_DIC
          : pre == "FDIC" ? CFX_PRE_FDIC
          : pre == "DILU" ? CFX_PRE_DILU
          : pre == "diagonal" ? CFX_PRE_DIAGONAL
          : pre == "GAMG" ? CFX_PRE_GAMG
          : CFX_PRE_NONE;
        // the GAMG keys: the solver's own, or the GAMG preconditioner's
        // (GAMGPreconditioner.C:40-79: nVcycles, its tolerance and relTol)
        const bool pcGamg =
            pd && c.preconditioner == CFX_PRE_GAMG
         && solverType != CFX_SOLVER_GAMG;
        const dictionary& gd = pcGamg ? *pd : controlDict_;
        if (pcGamg)
        {
            c.nVcycles = gd.lookupOrDefault<label>("nVcycles", 2);
            c.pcTolerance = gd.lookupOrDefault<scalar>("tolerance", 1e-6);
            c.pcRelTol = gd.lookupOrDefault<scalar>("relTol", 0);
        }
        // GAMG (GAMGSolver.C:67-93) and smoothSolver (smoothSolver.C:
        // 84-94) construct smoothers; the GAMG preconditioner's cycles too
        const bool smoothed =
            solverType == CFX_SOLVER_GAMG || solverType == CFX_SOLVER_SMOOTH
         || pcGamg;
        const word sm
        (
            smoothed ? smootherName(gd) : word("GaussSeidel")
        );
        c.smoother =
            sm == "DIC" ? CFX_SMOOTH_DIC
          : sm == "FDIC" ? CFX_SMOOTH_FDIC
          : sm == "nonBlockingGaussSeidel" ? CFX_SMOOTH_NBGS
          : sm == "symGaussSeidel" ? CFX_SMOOTH_SYMGS
          : sm == "DILU" ? CFX_SMOOTH_DILU
          : sm == "DICGaussSeidel" ? CFX_SMOOTH_DICGS
          : sm == "DILUGaussSeidel" ? CFX_SMOOTH_DILUGS
          : CFX_SMOOTH_GS;
        c.nSweeps = controlDict_.lookupOrDefault<label>("nSweeps", 1);
        c.nPreSweeps = gd.lookupOrDefault<label>("nPreSweeps", 0);
        c.preSweepsLevelMultiplier =
            gd.lookupOrDefault<label>("preSweepsLevelMultiplier", 1);
        c.maxPreSweeps = gd.lookupOrDefault<label>("maxPreSweeps", 4);
        c.nPostSweeps = gd.lookupOrDefault<label>("nPostSweeps", 2);
        c.postSweepsLevelMultiplier =
            gd.lookupOrDefault<label>("postSweepsLevelMultiplier", 1);
        c.maxPostSweeps = gd.lookupOrDefault<label>("maxPostSweeps", 4);
        c.nFinestSweeps = gd.lookupOrDefault<label>("nFinestSweeps", 2);
        c.scaleCorrection =
            gd.lookupOrDefault<bool>
            (
                "scaleCorrection", matrix_.symmetric()
            );
        c.interpolateCorrection =
            gd.lookupOrDefault<bool>("interpolateCorrection", false);
        c.directSolveCoarsest =
            gd.lookupOrDefault<bool>("directSolveCoarsest", false);
        const word precision
        (
            controlDict_.lookupOrDefault<word>("precision", "FP64")
        );
        if (precision != "FP64" && precision != "mixed")
        {
            FatalIOErrorInFunction(controlDict_)
                << "cudaLduSolvers: unknown precision " << precision
                << " (FP64 or mixed)" << exit(FatalIOError);
        }
        c.precision = precision == "mixed" ? CFX_MIXED : CFX_FP64;
        return c;
    }

    solverPerformance run
    (
        Entry& e,
        const cfx_controls& c,
        scalarField& psi,
        const scalarField& source
    ) const
    {
        cfx_perf perf;
        const int status =
            cfx_solve(e.mat, &c, psi.data(), source.cdata(), &perf);
        if (status == CFX_ERR_CONFIG)
        {
            FatalIOErrorInFunction(controlDict_)
                << cfx_last_error() << exit(FatalIOError);
        }
        check(status, "cfx_solve");

        solverPerformance sp(word(perf.solverName), fieldName_);
        sp.initialResidual() = perf.initialResidual;
        sp.finalResidual() = perf.finalResidual;
        sp.nIterations() = perf.nIterations;
        sp.checkConvergence(tolerance_, relTol_);
        if (perf.singular) sp.checkSingularity(0);
        return sp;
    }

public:

    cudaLduSolver
    (
        const word& fieldName,
        const lduMatrix& matrix,
        const Field<Field<scalar>>& interfaceBouCoeffs,
        const Field<Field<scalar>>& interfaceIntCoeffs,
        const lduInterfaceFieldPtrsList& interfaces,
        const dictionary& solverControls
    )
    :
        lduMatrix::solver
        (
            fieldName, matrix, interfaceBouCoeffs, interfaceIntCoeffs,
            interfaces, solverControls
        )
    {}
};


#define CUDA_LDU_SOLVER(Name, Type)                                            \
class Name                                                                     \
:                                                                              \
    public cudaLduSolver                                                       \
{                                                                              \
public:                                                                        \
    TypeName(#Name);                                                           \
    Name                                                                       \
    (                                                                          \
        const word& fieldName,                                                 \
        const lduMatrix& matrix,                                               \
        const Field<Field<scalar>>& interfaceBouCoeffs,                        \
        const Field<Field<scalar>>& interfaceIntCoeffs,                        \
        const lduInterfaceFieldPtrsList& interfaces,                           \
        const dictionary& solverControls                                       \
    )                                                                          \
    :                                                                          \
        cudaLduSolver                                                          \
        (                                                                      \
            fieldName, matrix, interfaceBouCoeffs, interfaceIntCoeffs,         \
            interfaces, solverControls                                         \
        )                                                                      \
    {}                                                                         \
    virtual solverPerformance solve                                            \
    (                                                                          \
        scalarField& psi,                                                      \
        const scalarField& source,                                             \
        const direction cmpt = 0                                               \
    ) const;                                                                   \
};

CUDA_LDU_SOLVER(cudaPCG, CFX_SOLVER_PCG)
CUDA_LDU_SOLVER(cudaPBiCGStab, CFX_SOLVER_PBICGSTAB)
CUDA_LDU_SOLVER(cudaGAMG, CFX_SOLVER_GAMG)
CUDA_LDU_SOLVER(cudaSmoothSolver, CFX_SOLVER_SMOOTH)
CUDA_LDU_SOLVER(cudaPBiCG, CFX_SOLVER_PBICG)

defineTypeNameAndDebug(cudaPCG, 0);
defineTypeNameAndDebug(cudaPBiCGStab, 0);
defineTypeNameAndDebug(cudaGAMG, 0);
defineTypeNameAndDebug(cudaSmoothSolver, 0);
defineTypeNameAndDebug(cudaPBiCG, 0);

lduMatrix::solver::addsymMatrixConstructorToTable<cudaPCG>
    addcudaPCGSymMatrixConstructorToTable_;
lduMatrix::solver::addsymMatrixConstructorToTable<cudaPBiCGStab>
    addcudaPBiCGStabSymMatrixConstructorToTable_;
lduMatrix::solver::addasymMatrixConstructorToTable<cudaPBiCGStab>
    addcudaPBiCGStabAsymMatrixConstructorToTable_;
lduMatrix::solver::addsymMatrixConstructorToTable<cudaGAMG>
    addcudaGAMGSymMatrixConstructorToTable_;
lduMatrix::solver::addasymMatrixConstructorToTable<cudaGAMG>
    addcudaGAMGAsymMatrixConstructorToTable_;
lduMatrix::solver::addsymMatrixConstructorToTable<cudaSmoothSolver>
    addcudaSmoothSolverSymMatrixConstructorToTable_;
lduMatrix::solver::addasymMatrixConstructorToTable<cudaSmoothSolver>
    addcudaSmoothSolverAsymMatrixConstructorToTable_;
// PBiCG.C:34-35: asymmetric matrices only
lduMatrix::solver::addasymMatrixConstructorToTable<cudaPBiCG>
    addcudaPBiCGAsymMatrixConstructorToTable_;


solverPerformance cudaPCG::solve
(
    scalarField& psi,
    const scalarField& source,
    const direction
) const
{
    const cfx_controls c = controls(CFX_SOLVER_PCG);
    Entry& e = deviceMatrix();
    if (c.preconditioner == CFX_PRE_GAMG) gamgLevels(e, *preconditionerDict());
    return run(e, c, psi, source);
}


solverPerformance cudaPBiCGStab::solve
(
    scalarField& psi,
    const scalarField& source,
    const direction
) const
{
    const cfx_controls c = controls(CFX_SOLVER_PBICGSTAB);
    Entry& e = deviceMatrix();
    if (c.preconditioner == CFX_PRE_GAMG) gamgLevels(e, *preconditionerDict());
    return run(e, c, psi, source);
}


solverPerformance cudaPBiCG::solve
(
    scalarField& psi,
    const scalarField& source,
    const direction
) const
{
    const cfx_controls c = controls(CFX_SOLVER_PBICG);
    Entry& e = deviceMatrix();
    return run(e, c, psi, source);
}


solverPerformance cudaSmoothSolver::solve
(
    scalarField& psi,
    const scalarField& source,
    const direction
) const
{
    const cfx_controls c = controls(CFX_SOLVER_SMOOTH);
    Entry& e = deviceMatrix();
    return run(e, c, psi, source);
}


solverPerformance cudaGAMG::solve
(
    scalarField& psi,
    const scalarField& source,
    const direction
) const
{
    const cfx_controls c = controls(CFX_SOLVER_GAMG);
    Entry& e = deviceMatrix();
    gamgLevels(e, controlDict_);
    return run(e, c, psi, source);
}

} // End namespace Foam
