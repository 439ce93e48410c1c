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
  solve.  Coupled interfaces are not supported: a matrix with any set
  interface is refused with FatalError.
\*---------------------------------------------------------------------------*/

#include "lduMatrix.H"
#include "GAMGAgglomeration.H"
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
        forAll(interfaces_, patchi)
        {
            if (interfaces_.set(patchi))
            {
                FatalErrorInFunction
                    << "cudaLduSolvers: coupled interfaces are not supported"
                    << exit(FatalError);
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
        return e;
    }

    cfx_controls controls(int solverType) const
    {
        cfx_controls c;
        cfx_default_controls(&c);
        c.solver = solverType;
        c.tolerance = tolerance_;
        c.relTol = relTol_;
        c.maxIter = maxIter_;
        c.minIter = minIter_;
        const word pre
        (
            controlDict_.lookupOrDefault<word>("preconditioner", "none")
        );
        c.preconditioner =
            pre == "DIC" ? CFX_PRE_DIC
          : pre == "DILU" ? CFX_PRE_DILU
          : pre == "diagonal" ? CFX_PRE_DIAGONAL
          : CFX_PRE_NONE;
        const word sm
        (
            controlDict_.lookupOrDefault<word>("smoother", "GaussSeidel")
        );
        c.smoother =
            sm == "DIC" ? CFX_SMOOTH_DIC
          : sm == "symGaussSeidel" ? CFX_SMOOTH_SYMGS
          : sm == "DILU" ? CFX_SMOOTH_DILU
          : sm == "DICGaussSeidel" ? CFX_SMOOTH_DICGS
          : sm == "DILUGaussSeidel" ? CFX_SMOOTH_DILUGS
          : CFX_SMOOTH_GS;
        c.nSweeps = controlDict_.lookupOrDefault<label>("nSweeps", 1);
        c.nPreSweeps = controlDict_.lookupOrDefault<label>("nPreSweeps", 0);
        c.preSweepsLevelMultiplier =
            controlDict_.lookupOrDefault<label>("preSweepsLevelMultiplier", 1);
        c.maxPreSweeps = controlDict_.lookupOrDefault<label>("maxPreSweeps", 4);
        c.nPostSweeps = controlDict_.lookupOrDefault<label>("nPostSweeps", 2);
        c.postSweepsLevelMultiplier =
            controlDict_.lookupOrDefault<label>("postSweepsLevelMultiplier", 1);
        c.maxPostSweeps = controlDict_.lookupOrDefault<label>("maxPostSweeps", 4);
        c.nFinestSweeps = controlDict_.lookupOrDefault<label>("nFinestSweeps", 2);
        c.scaleCorrection =
            controlDict_.lookupOrDefault<bool>
            (
                "scaleCorrection", matrix_.symmetric()
            );
        c.precision =
            controlDict_.lookupOrDefault<word>("precision", "FP64") == "mixed"
          ? CFX_MIXED : CFX_FP64;
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

defineTypeNameAndDebug(cudaPCG, 0);
defineTypeNameAndDebug(cudaPBiCGStab, 0);
defineTypeNameAndDebug(cudaGAMG, 0);
defineTypeNameAndDebug(cudaSmoothSolver, 0);

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


solverPerformance cudaPCG::solve
(
    scalarField& psi,
    const scalarField& source,
    const direction
) const
{
    Entry& e = deviceMatrix();
    return run(e, controls(CFX_SOLVER_PCG), psi, source);
}


solverPerformance cudaPBiCGStab::solve
(
    scalarField& psi,
    const scalarField& source,
    const direction
) const
{
    Entry& e = deviceMatrix();
    return run(e, controls(CFX_SOLVER_PBICGSTAB), psi, source);
}


solverPerformance cudaSmoothSolver::solve
(
    scalarField& psi,
    const scalarField& source,
    const direction
) const
{
    Entry& e = deviceMatrix();
    return run(e, controls(CFX_SOLVER_SMOOTH), psi, source);
}


solverPerformance cudaGAMG::solve
(
    scalarField& psi,
    const scalarField& source,
    const direction
) const
{
    Entry& e = deviceMatrix();
    if (!e.gamg)
    {
        // The reference's own agglomeration (faceAreaPair on an fvMesh),
        // cached in the mesh registry (GAMGAgglomeration.C:349-400); its
        // restriction maps define the device hierarchy.
        const GAMGAgglomeration& agg =
            GAMGAgglomeration::New(matrix_, controlDict_);
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
    return run(e, controls(CFX_SOLVER_GAMG), psi, source);
}

} // End namespace Foam
