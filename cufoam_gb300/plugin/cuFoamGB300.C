/*
 * cuFoamGB300.C -- implementation of the eight plugins (see cuFoamGB300.H).
 *
 * What one solve() does, compared with the reference's plugin
 * (cuFoamCG/cuFoamCG.C:38-90):
 *   reference: host ldu2csr, cudaMalloc+copy of the CSR and vectors,
 *              NormFactor, the solver with tolerance*normFactor, copy back,
 *              free everything.
 *   here:      the lduAddressing is uploaded once and kept on the device
 *              (an LRU cache of four meshes, keyed on the addressing's
 *              memory, sizes and a sampled fingerprint of its contents);
 *              each call uploads the
 *              coefficients, converts them on the device, and runs
 *              normFactor + the solver inside one device-driven loop.
 * Meshes with cyclic patches solve on a coupled matrix (the interface
 * coefficients appended to their rows), kept in a cache of its own whose
 * values are refreshed on every solve.
 * Fixed relative to the reference: the constructor forwards
 * interfaceBouCoeffs (the reference passes interfaceIntCoeffs twice,
 * cuFoamCG/cuFoamCG.C:30-31).
 * In a parallel run each rank solves its subdomain through
 * cf_solve_decomposed, the processor patches exchanged by OpenFOAM's own
 * Pstream (cuFoamGB300Comm.H); the reference solves each subdomain alone.
 */
#include "cuFoamGB300.H"
#include "cuFoamGB300Comm.H"

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

namespace Foam {

namespace {

// One lock for the plugin's shared state: the context (one host thread at a
// time) and the matrix cache.  solve() holds it from the matrix lookup to
// the end of cf_solve.
std::mutex &gb300Mutex()
{
    static std::mutex m;
    return m;
}

cf_context *gb300Context()
{
    static cf_context *ctx = nullptr;
    if (!ctx) {
        const char *dev = std::getenv("CUFOAM_GB300_DEVICE");
        const int device = dev ? std::atoi(dev) : 0;
        const cf_status st = cf_context_create(device, &ctx);
        if (st != CF_OK) {
            FatalErrorInFunction << "cuFoamGB300: cannot open CUDA device " << device << ": "
                                 << cf_status_string(st) << exit(FatalError);
        }
    }
    return ctx;
}

// FNV-1a over the sizes and a fixed sample of the owner / neighbour lists
// (their first and last 256 entries and 4,096 evenly spaced ones): a few
// microseconds, and a new mesh that reuses an old one's memory (same
// pointers, same sizes, other faces) gives another value.
uint64_t addressingFingerprint(const lduAddressing &A, label n)
{
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](uint64_t v) {
        for (int k = 0; k < 8; ++k) {
            h ^= (v >> (8 * k)) & 0xffu;
            h *= 1099511628211ull;
        }
    };
    const labelList &la = A.lowerAddr(), &ua = A.upperAddr();
    const label nf = la.size();
    mix((uint64_t)n);
    mix((uint64_t)nf);
    auto sample = [&](label f) {
        mix((uint64_t)(uint32_t)la[f]);
        mix((uint64_t)(uint32_t)ua[f]);
    };
    const label edge = nf < 256 ? nf : 256;
    for (label f = 0; f < edge; ++f) sample(f);
    for (label f = nf - edge; f < nf; ++f) sample(f);
    if (nf > 0)
        for (label k = 0; k < 4096; ++k) sample((label)(((int64_t)k * nf) / 4096));
    return h;
}

// Device matrices kept across solve() calls: reused by Ux/Uy/Uz and across
// time steps (coefficients refreshed on every solve), a few meshes at a time
// (multi-region cases), the least recently used dropped first.  An entry
// matches on the addressing lists' memory, the sizes and the fingerprint,
// so a mesh that replaced another in the same memory is rebuilt.
struct MatrixCacheEntry {
    const void *lowerAddr = nullptr;
    const void *upperAddr = nullptr;
    label n = -1, nFaces = -1;
    uint64_t fingerprint = 0;
    uint64_t lastUse = 0;
    cf_matrix *m = nullptr;
};

constexpr size_t kMatrixCacheEntries = 4;
std::vector<MatrixCacheEntry> gMatrixCache;
uint64_t gMatrixClock = 0;
long gMatrixBuilds = 0;

cf_matrix *deviceMatrix(const lduMatrix &M)   // under gb300Mutex()
{
    const lduAddressing &A = M.lduAddr();
    const label n = M.diag().size();
    const label nFaces = A.lowerAddr().size();
    const uint64_t fp = addressingFingerprint(A, n);
    cf_context *ctx = gb300Context();
    MatrixCacheEntry *hit = nullptr, *stale = nullptr;
    for (MatrixCacheEntry &e : gMatrixCache) {
        const bool same_memory = e.lowerAddr == A.lowerAddr().cdata() && e.upperAddr == A.upperAddr().cdata();
        if (same_memory && e.n == n && e.nFaces == nFaces && e.fingerprint == fp) hit = &e;
        else if (same_memory) stale = &e;   // other faces in the same memory: rebuild
    }
    cf_status st = CF_OK;
    if (hit) {
        st = cf_matrix_update_values(hit->m, M.diag().cdata(), M.lower().cdata(), M.upper().cdata(),
                                     CF_MEM_HOST);
    } else {
        MatrixCacheEntry *slot = stale;
        if (!slot && gMatrixCache.size() < kMatrixCacheEntries) {
            gMatrixCache.reserve(kMatrixCacheEntries);
            gMatrixCache.emplace_back();
            slot = &gMatrixCache.back();
        }
        if (!slot) {
            slot = &gMatrixCache[0];
            for (MatrixCacheEntry &e : gMatrixCache)
                if (e.lastUse < slot->lastUse) slot = &e;
        }
        if (slot->m) cf_matrix_destroy(slot->m);
        *slot = MatrixCacheEntry();
        cf_ldu_view v;
        std::memset(&v, 0, sizeof(v));
        v.n_cells = n;
        v.n_faces = nFaces;
        v.diag = M.diag().cdata();
        v.lower = M.lower().cdata();
        v.upper = M.upper().cdata();
        v.lower_addr = A.lowerAddr().cdata();
        v.upper_addr = A.upperAddr().cdata();
        v.losort = A.losortAddr().cdata();
        v.losort_start = A.losortStartAddr().cdata();
        v.owner_start = A.ownerStartAddr().cdata();
        v.memory = CF_MEM_HOST;
        st = cf_matrix_create_ldu(ctx, &v, &slot->m);
        if (st == CF_OK) {
            slot->lowerAddr = A.lowerAddr().cdata();
            slot->upperAddr = A.upperAddr().cdata();
            slot->n = n;
            slot->nFaces = nFaces;
            slot->fingerprint = fp;
            ++gMatrixBuilds;
            hit = slot;
        }
    }
    if (st != CF_OK) {
        FatalErrorInFunction << "cuFoamGB300: cannot load the matrix: " << cf_status_string(st)
                             << ": " << cf_context_last_error(ctx) << exit(FatalError);
    }
    hit->lastUse = ++gMatrixClock;
    return hit->m;
}

// Coupled matrices (cyclic patches folded in), kept across solve() calls
// like the device matrices: keyed on the addressing (as above) and on the
// cyclic patches' face cells, all of them hashed.  Each entry holds, for
// every CSR entry, where its value comes from in [diag | lower | upper | the
// interface coefficients in patch and face order], so a repeat solve
// gathers its values on the host and refreshes them on the device
// (cf_matrix_update_csr_values): no conversion, no allocation, no SELL-32
// layout rebuild.
struct CoupledCacheEntry {
    const void *lowerAddr = nullptr;
    const void *upperAddr = nullptr;
    label n = -1, nFaces = -1;
    uint64_t fingerprint = 0, ifcFingerprint = 0;
    uint64_t lastUse = 0;
    cf_matrix *m = nullptr;
    std::vector<int32_t> src;   // value source of each CSR entry
    std::vector<double> vals;   // the gathered values
};

std::vector<CoupledCacheEntry> gCoupledCache;
long gCoupledBuilds = 0;

} // namespace

static_assert(sizeof(label) == sizeof(int32_t), "cuFoamGB300 needs 32-bit labels");
static_assert(sizeof(scalar) == sizeof(double), "cuFoamGB300 needs double scalars");

cuFoamGB300Solver::cuFoamGB300Solver(int32_t kind, const word &fieldName, const lduMatrix &matrix,
                                     const FieldField<Field, scalar> &interfaceBouCoeffs,
                                     const FieldField<Field, scalar> &interfaceIntCoeffs,
                                     const lduInterfaceFieldPtrsList &interfaces,
                                     const dictionary &solverControls)
    : lduMatrix::solver(fieldName, matrix, interfaceBouCoeffs, interfaceIntCoeffs, interfaces,
                        solverControls),
      kind_(kind)
{
}

cf_controls cuFoamGB300Solver::gb300Controls() const
{
    cf_controls c;
    cf_controls_init(&c);
    c.tolerance = tolerance_;
    c.max_iter = maxIter_;
    const dictionary &d = controlDict();
    if (d.lookupOrDefault<bool>("useRelTol", false)) {
        c.rel_tol = relTol_;
        c.min_iter = minIter_;
    }
    const word precision = d.lookupOrDefault<word>("precision", word("FP64"));
    c.precision = (precision == "mixed") ? CF_PREC_MIXED : CF_PREC_FP64;
    // "auto" (default): the reference's summation order for BiCG, the fast
    // one for the others
    const word reduction = d.lookupOrDefault<word>("reduction", word("auto"));
    c.reduction = (reduction == "reference") ? CF_REDUCE_REFERENCE
                  : (reduction == "fast")    ? CF_REDUCE_FAST
                                             : CF_REDUCE_AUTO;
    const word normType = d.lookupOrDefault<word>("normType", word("reference"));
    c.norm_type = (normType == "openfoam") ? CF_NORM_OPENFOAM_L1 : CF_NORM_REFERENCE_L2;
    c.memory = CF_MEM_HOST;
    return c;
}

cf_matrix *cuFoamGB300Solver::coupledMatrix() const   // under gb300Mutex()
{
    // couplings of the cyclic patches: (faceCell, neighbour faceCell,
    // -coeff), numbered in patch and face order
    struct Extra {
        label col;
        int32_t e;
    };
    std::vector<std::vector<Extra>> extra;
    std::vector<double> ext;   // -coeff of extra e
    uint64_t ifp = 1469598103934665603ull;
    auto mix = [&ifp](uint64_t v) {
        for (int k = 0; k < 8; ++k) {
            ifp ^= (v >> (8 * k)) & 0xffu;
            ifp *= 1099511628211ull;
        }
    };
    const lduInterfaceFieldPtrsList &ifs = interfaces();
    for (label patchi = 0; patchi < ifs.size(); ++patchi) {
        if (!ifs.set(patchi)) continue;
        const lduInterface &ifc = ifs[patchi].interface();
        if (isA<processorLduInterface>(ifc)) continue;   // solve(): the decomposed path
        if (!isA<cyclicLduInterface>(ifc)) {
            FatalErrorInFunction << type() << ": patch " << patchi
                                 << " is a coupled interface other than cyclic or processor; "
                                    "only those two are solved on the GPU"
                                 << exit(FatalError);
        }
        const cyclicLduInterface &cyc = refCast<const cyclicLduInterface>(ifc);
        const labelList &fc = cyc.faceCells();
        const labelList &nfc = cyc.neighbPatch().faceCells();
        const scalarField &coeffs = interfaceBouCoeffs()[patchi];
        if (nfc.size() != fc.size() || coeffs.size() != fc.size()) {
            FatalErrorInFunction << type() << ": cyclic patch " << patchi
                                 << " does not match its neighbour" << exit(FatalError);
        }
        if (extra.empty()) extra.resize(matrix().diag().size());
        mix((uint64_t)patchi);
        mix((uint64_t)fc.size());
        for (label f = 0; f < fc.size(); ++f) {
            mix((uint64_t)(uint32_t)fc[f]);
            mix((uint64_t)(uint32_t)nfc[f]);
            extra[fc[f]].push_back({nfc[f], (int32_t)ext.size()});
            ext.push_back(-coeffs[f]);
        }
    }
    if (ext.empty()) return nullptr;
    const lduMatrix &M = matrix();
    const lduAddressing &A = M.lduAddr();
    const label n = M.diag().size(), nf = A.lowerAddr().size();
    const uint64_t fp = addressingFingerprint(A, n);
    cf_context *ctx = gb300Context();
    CoupledCacheEntry *hit = nullptr, *slot = nullptr;
    for (CoupledCacheEntry &e : gCoupledCache) {
        if (e.lowerAddr == A.lowerAddr().cdata() && e.upperAddr == A.upperAddr().cdata() && e.n == n &&
            e.nFaces == nf && e.fingerprint == fp && e.ifcFingerprint == ifp)
            hit = &e;
    }
    cf_status st = CF_OK;
    if (!hit) {
        // the LDU part as the reference's CSR (device ldu2csr) on
        // index-encoded values: each entry's value is its source position
        std::vector<double> di((size_t)n), lo((size_t)nf), up((size_t)nf);
        for (label i = 0; i < n; ++i) di[(size_t)i] = (double)i;
        for (label f = 0; f < nf; ++f) {
            lo[(size_t)f] = (double)(n + f);
            up[(size_t)f] = (double)(n + nf + f);
        }
        cf_ldu_view v;
        std::memset(&v, 0, sizeof(v));
        v.n_cells = n;
        v.n_faces = nf;
        v.diag = di.data();
        v.lower = lo.data();
        v.upper = up.data();
        v.lower_addr = A.lowerAddr().cdata();
        v.upper_addr = A.upperAddr().cdata();
        v.losort = A.losortAddr().cdata();
        v.losort_start = A.losortStartAddr().cdata();
        v.owner_start = A.ownerStartAddr().cdata();
        v.memory = CF_MEM_HOST;
        std::vector<int32_t> ro((size_t)n + 1), col((size_t)n + 2 * (size_t)nf);
        std::vector<double> pos(col.size());
        st = cf_ldu2csr(ctx, &v, ro.data(), col.data(), pos.data(), CF_MEM_HOST);
        if (st == CF_OK) {
            // then each row's interface entries after its own
            if (gCoupledCache.size() < kMatrixCacheEntries) {
                gCoupledCache.reserve(kMatrixCacheEntries);
                gCoupledCache.emplace_back();
                slot = &gCoupledCache.back();
            } else {
                slot = &gCoupledCache[0];
                for (CoupledCacheEntry &e : gCoupledCache)
                    if (e.lastUse < slot->lastUse) slot = &e;
            }
            if (slot->m) cf_matrix_destroy(slot->m);
            *slot = CoupledCacheEntry();
            std::vector<int32_t> ro2((size_t)n + 1), col2;
            col2.reserve(col.size() + ext.size());
            slot->src.reserve(col.size() + ext.size());
            for (label i = 0; i < n; ++i) {
                ro2[(size_t)i] = (int32_t)col2.size();
                for (int32_t j = ro[(size_t)i]; j < ro[(size_t)i + 1]; ++j) {
                    col2.push_back(col[(size_t)j]);
                    slot->src.push_back((int32_t)pos[(size_t)j]);
                }
                for (const Extra &x : extra[(size_t)i]) {
                    col2.push_back(x.col);
                    slot->src.push_back((int32_t)(n + 2 * nf) + x.e);
                }
            }
            ro2[(size_t)n] = (int32_t)col2.size();
            slot->vals.resize(col2.size());
            hit = slot;
            ++gCoupledBuilds;
            // values gathered below, then the matrix made from them
            std::vector<int32_t>().swap(ro);
            std::vector<int32_t>().swap(col);
            slot->lowerAddr = A.lowerAddr().cdata();
            slot->upperAddr = A.upperAddr().cdata();
            slot->n = n;
            slot->nFaces = nf;
            slot->fingerprint = fp;
            slot->ifcFingerprint = ifp;
            const scalar *d = M.diag().cdata(), *l = M.lower().cdata(), *u = M.upper().cdata();
            for (size_t j = 0; j < slot->src.size(); ++j) {
                const int32_t q = slot->src[j];
                slot->vals[j] = q < n ? d[q] : q < n + nf ? l[q - n] : q < n + 2 * nf ? u[q - n - nf]
                                                                                  : ext[(size_t)(q - n - 2 * nf)];
            }
            st = cf_matrix_create_csr(ctx, n, (int64_t)col2.size(), ro2.data(), col2.data(), slot->vals.data(),
                                      CF_MEM_HOST, &slot->m);
            if (st != CF_OK) {
                slot->m = nullptr;
                *slot = CoupledCacheEntry();
            }
        }
    } else {
        // the same pattern: this call's coefficients in the cached order
        const scalar *d = M.diag().cdata(), *l = M.lower().cdata(), *u = M.upper().cdata();
        for (size_t j = 0; j < hit->src.size(); ++j) {
            const int32_t q = hit->src[j];
            hit->vals[j] = q < n ? d[q] : q < n + nf ? l[q - n] : q < n + 2 * nf ? u[q - n - nf]
                                                                              : ext[(size_t)(q - n - 2 * nf)];
        }
        st = cf_matrix_update_csr_values(hit->m, hit->vals.data(), CF_MEM_HOST);
    }
    if (st != CF_OK || !hit || !hit->m) {
        FatalErrorInFunction << "cuFoamGB300: cannot load the coupled matrix: " << cf_status_string(st)
                             << ": " << cf_context_last_error(ctx) << exit(FatalError);
    }
    hit->lastUse = ++gMatrixClock;
    return hit->m;
}

solverPerformance cuFoamGB300Solver::solve(scalarField &psi, const scalarField &source,
                                           const direction) const
{
    std::lock_guard<std::mutex> lock(gb300Mutex());
    // processor patches: this matrix is one subdomain of a decomposed case
    const cuFoamGB300ProcessorComm procs(interfaces(), interfaceBouCoeffs());
    const bool decomposed = Pstream::parRun();
    if (!decomposed && procs.nPatches() > 0) {
        FatalErrorInFunction << type() << ": processor patches outside a parallel run"
                             << exit(FatalError);
    }
    cf_matrix *coupled = coupledMatrix();
    cf_matrix *m = coupled ? coupled : deviceMatrix(matrix());
    const cf_controls c = gb300Controls();
    cf_perf perf;
    std::memset(&perf, 0, sizeof(perf));
    cf_status st;
    if (decomposed) {
        // every rank takes part, with or without processor faces: the
        // normFactor and the inner products are sums over all ranks
        const cf_interfaces ifc = procs.interfaces();
        const cf_comm comm = procs.comm();
        st = cf_solve_decomposed(m, kind_, &c, &ifc, &comm, source.cdata(), psi.data(), &perf);
    } else {
        st = cf_solve(m, kind_, &c, source.cdata(), psi.data(), &perf);
    }
    if (st != CF_OK) {
        FatalErrorInFunction << type() << ": solve failed: " << cf_status_string(st) << ": "
                             << cf_context_last_error(gb300Context()) << exit(FatalError);
    }
    solverPerformance solverPerf(type(), fieldName());
    solverPerf.initialResidual() = perf.initial_residual;
    solverPerf.finalResidual() = perf.final_residual;
    solverPerf.nIterations() = perf.n_iterations;
    solverPerf.checkConvergence(tolerance_, relTol_);
    return solverPerf;
}

// ---------------------------------------------------------------------------
// the eight plugins and their run-time selection entries.  CG and
// Richardson register for symmetric matrices only, as the reference's do
// (cuFoamCG/cuFoamCG.C:14-15, cuFoamRichardson/cuFoamRichardson.C:11-12).
// ---------------------------------------------------------------------------
#define CUFOAM_GB300_DEFINE_SOLVER(Name, Kind)                                               \
    defineTypeNameAndDebug(Name, 0);                                                         \
    Name::Name(const word &fieldName, const lduMatrix &matrix,                               \
               const FieldField<Field, scalar> &interfaceBouCoeffs,                          \
               const FieldField<Field, scalar> &interfaceIntCoeffs,                          \
               const lduInterfaceFieldPtrsList &interfaces, const dictionary &solverControls) \
        : cuFoamGB300Solver(Kind, fieldName, matrix, interfaceBouCoeffs, interfaceIntCoeffs, \
                            interfaces, solverControls)                                      \
    {                                                                                        \
    }                                                                                        \
    lduMatrix::solver::addsymMatrixConstructorToTable<Name> add##Name##SymMatrixConstructorToTable_;

#define CUFOAM_GB300_ASYMMETRIC(Name)                                                        \
    lduMatrix::solver::addasymMatrixConstructorToTable<Name> add##Name##AsymMatrixConstructorToTable_;

CUFOAM_GB300_DEFINE_SOLVER(cuFoamCG, CF_CG)
CUFOAM_GB300_DEFINE_SOLVER(cuFoamBiCG, CF_BICG)
CUFOAM_GB300_ASYMMETRIC(cuFoamBiCG)
CUFOAM_GB300_DEFINE_SOLVER(cuFoamJacobi, CF_JACOBI)
CUFOAM_GB300_ASYMMETRIC(cuFoamJacobi)
CUFOAM_GB300_DEFINE_SOLVER(cuFoamMR, CF_MR)
CUFOAM_GB300_ASYMMETRIC(cuFoamMR)
CUFOAM_GB300_DEFINE_SOLVER(cuFoamMRJacobi, CF_MRJACOBI)
CUFOAM_GB300_ASYMMETRIC(cuFoamMRJacobi)
CUFOAM_GB300_DEFINE_SOLVER(cuFoamMRS, CF_MRS)
CUFOAM_GB300_ASYMMETRIC(cuFoamMRS)
CUFOAM_GB300_DEFINE_SOLVER(cuFoamJMR, CF_JMR)
CUFOAM_GB300_ASYMMETRIC(cuFoamJMR)
CUFOAM_GB300_DEFINE_SOLVER(cuFoamRichardson, CF_RICHARDSON)
// Jacobi-preconditioned CG (no reference counterpart), symmetric matrices
CUFOAM_GB300_DEFINE_SOLVER(cuFoamPCG, CF_PCG)

} // namespace Foam

// Device matrices the plugin has built since the library was loaded (a
// diagnostic for tests of the matrix cache).
extern "C" long cuFoamGB300_matrix_builds()
{
    std::lock_guard<std::mutex> lock(Foam::gb300Mutex());
    return Foam::gMatrixBuilds;
}

// Coupled (cyclic) matrices the plugin has built since the library was
// loaded (a diagnostic for tests of their cache).
extern "C" long cuFoamGB300_coupled_builds()
{
    std::lock_guard<std::mutex> lock(Foam::gb300Mutex());
    return Foam::gCoupledBuilds;
}
