/*
 * minifoam_harness.C -- drives the plugin sources the way OpenFOAM does,
 * without OpenFOAM: builds an lduAddressing/lduMatrix from plain arrays,
 * selects the solver by name from the run-time tables
 * (lduMatrix::solver::New) and calls solve(psi, source, cmpt).  Exposed as
 * a C function so the tests can exercise the plugin layer end to end.
 */
#include "lduMatrix.H"
#include "../cuFoamGB300Comm.H"

#include <cstring>
#include <exception>
#include <map>
#include <memory>

namespace Foam {
FatalErrorType FatalError;
}

namespace {

// One cyclic patch pair (faces of patch A coupled to patch B, and back),
// an optional processor patch; n_cyc = 0: no interfaces.  Processor
// patches of a decomposed case: n_proc patches, patch p to rank
// proc_neighbour[p] with proc_size[p] faces; their face cells and
// interfaceBouCoeffs patch after patch.
struct Coupling {
    int n_cyc = 0;
    const int *fcA = nullptr, *fcB = nullptr;
    const double *coeffA = nullptr, *coeffB = nullptr;
    bool processor = false;
    int n_proc = 0;
    const int *proc_neighbour = nullptr, *proc_size = nullptr, *proc_cells = nullptr;
    const double *proc_coeffs = nullptr;
};

// the processor interfaces of `cpl` appended to an interface list
struct ProcessorPatches {
    std::vector<std::unique_ptr<Foam::processorLduInterface>> patches;
    std::vector<std::unique_ptr<Foam::lduInterfaceField>> fields;

    void add(const Coupling &cpl, Foam::FieldField<Foam::Field, Foam::scalar> &bou,
             Foam::FieldField<Foam::Field, Foam::scalar> &intc, Foam::lduInterfaceFieldPtrsList &interfaces)
    {
        using namespace Foam;
        int o = 0;
        std::map<int, int> per_neighbour;   // the k-th patch to a rank: tag k + 1
        for (int p = 0; p < cpl.n_proc; ++p) {
            const int m = cpl.proc_size[p];
            const int tag = ++per_neighbour[cpl.proc_neighbour[p]];
            patches.emplace_back(new processorLduInterface(labelList(cpl.proc_cells + o, cpl.proc_cells + o + m),
                                                           cpl.proc_neighbour[p], tag));
            fields.emplace_back(new lduInterfaceField(*patches.back()));
            interfaces.push_back(fields.back().get());
            bou.push_back(scalarField(cpl.proc_coeffs + o, cpl.proc_coeffs + o + m));
            intc.push_back(scalarField(cpl.proc_coeffs + o, cpl.proc_coeffs + o + m));
            o += m;
        }
    }
};

// addressing objects (four slots) whose lists keep their memory between
// calls, like the meshes of a running case
Foam::lduAddressing *reusedAddressing(int slot, int n, const Foam::labelList &la, const Foam::labelList &ua)
{
    static Foam::lduAddressing *a[4] = {nullptr, nullptr, nullptr, nullptr};
    Foam::lduAddressing *&p = a[slot & 3];
    if (!p) p = new Foam::lduAddressing(n, la, ua);
    else p->reset(n, la, ua);
    return p;
}

int run(const char *solver_name, int n, int n_faces, const double *diag, const double *lower,
        const double *upper, const int *lower_addr, const int *upper_addr, const double *source,
        double *psi, double tolerance, double rel_tol, int max_iter, int n_extra, const char *const *keys,
        const char *const *values, const Coupling &cpl, double *out, char *err, int err_len,
        int reuse_slot = -1)
{
    try {
        using namespace Foam;
        labelList la(lower_addr, lower_addr + n_faces), ua(upper_addr, upper_addr + n_faces);
        std::unique_ptr<lduAddressing> own;
        if (reuse_slot < 0) own.reset(new lduAddressing(n, la, ua));
        const lduAddressing &addr = reuse_slot >= 0 ? *reusedAddressing(reuse_slot, n, la, ua) : *own;
        scalarField d(diag, diag + n), up(upper, upper + n_faces);
        scalarField lo;
        if (lower) lo.assign(lower, lower + n_faces);
        lduMatrix matrix(addr, d, lower ? &lo : nullptr, &up);
        dictionary controls;
        controls.set("solver", solver_name);
        {
            // exact text of the doubles
            char buf[64];
            std::snprintf(buf, sizeof(buf), "%.17g", tolerance);
            controls.set("tolerance", buf);
            std::snprintf(buf, sizeof(buf), "%.17g", rel_tol);
            controls.set("relTol", buf);
        }
        controls.set("maxIter", std::to_string(max_iter));
        for (int i = 0; i < n_extra; ++i) controls.set(keys[i], values[i]);
        FieldField<Field, scalar> bou, intc;
        lduInterfaceFieldPtrsList interfaces;
        // patch 0: an uncoupled wall; patches 1, 2: the cyclic pair; 3: processor
        std::unique_ptr<cyclicLduInterface> cycA, cycB;
        std::unique_ptr<processorLduInterface> proc;
        std::vector<std::unique_ptr<lduInterfaceField>> fields;
        bou.resize(1);
        intc.resize(1);
        interfaces.push_back(nullptr);
        if (cpl.n_cyc > 0) {
            cycA.reset(new cyclicLduInterface(labelList(cpl.fcA, cpl.fcA + cpl.n_cyc)));
            cycB.reset(new cyclicLduInterface(labelList(cpl.fcB, cpl.fcB + cpl.n_cyc)));
            cycA->setNeighbPatch(*cycB);
            cycB->setNeighbPatch(*cycA);
            fields.emplace_back(new lduInterfaceField(*cycA));
            fields.emplace_back(new lduInterfaceField(*cycB));
            interfaces.push_back(fields[0].get());
            interfaces.push_back(fields[1].get());
            bou.push_back(scalarField(cpl.coeffA, cpl.coeffA + cpl.n_cyc));
            bou.push_back(scalarField(cpl.coeffB, cpl.coeffB + cpl.n_cyc));
            intc.push_back(scalarField(cpl.coeffA, cpl.coeffA + cpl.n_cyc));
            intc.push_back(scalarField(cpl.coeffB, cpl.coeffB + cpl.n_cyc));
        }
        ProcessorPatches procs;
        procs.add(cpl, bou, intc, interfaces);
        if (cpl.processor) {
            proc.reset(new processorLduInterface(labelList(1, 0)));
            fields.emplace_back(new lduInterfaceField(*proc));
            interfaces.push_back(fields.back().get());
            bou.push_back(scalarField(1, 1.0));
            intc.push_back(scalarField(1, 1.0));
        }
        std::unique_ptr<lduMatrix::solver> s =
            lduMatrix::solver::New("psi", matrix, bou, intc, interfaces, controls);
        scalarField x(psi, psi + n), b(source, source + n);
        solverPerformance perf = s->solve(x, b);
        std::memcpy(psi, x.cdata(), sizeof(double) * n);
        out[0] = perf.initialResidual();
        out[1] = perf.finalResidual();
        out[2] = perf.nIterations();
        out[3] = perf.converged() ? 1.0 : 0.0;
        if (err && err_len > 0) err[0] = 0;
        return 0;
    } catch (const std::exception &e) {
        if (err && err_len > 0) {
            std::strncpy(err, e.what(), err_len - 1);
            err[err_len - 1] = 0;
        }
        return -1;
    }
}

} // namespace

extern "C" {

/* Solve with the plugin `solver_name` ("cuFoamCG", ...).  lower == NULL
 * means a symmetric matrix (OpenFOAM stores only upper then).  `keys` /
 * `values` are n_extra extra dictionary entries (e.g. "precision" "mixed").
 * out = {initialResidual, finalResidual, nIterations, converged}.
 * Returns 0, or -1 with the FatalError text in err. */
int mf_solve(const char *solver_name, int n, int n_faces, const double *diag, const double *lower,
             const double *upper, const int *lower_addr, const int *upper_addr, const double *source,
             double *psi, double tolerance, double rel_tol, int max_iter, int n_extra,
             const char *const *keys, const char *const *values, double *out, char *err, int err_len)
{
    return run(solver_name, n, n_faces, diag, lower, upper, lower_addr, upper_addr, source, psi, tolerance,
               rel_tol, max_iter, n_extra, keys, values, Coupling(), out, err, err_len);
}

/* mf_solve on the lduAddressing object of `slot` (0..3), kept between
 * calls with its lists overwritten in place: the same mesh across calls, or
 * a new mesh in an old mesh's memory (same addresses, and the same sizes
 * when the meshes match). */
int mf_solve_reused_addressing(int slot, const char *solver_name, int n, int n_faces, const double *diag,
                               const double *lower, const double *upper, const int *lower_addr,
                               const int *upper_addr, const double *source, double *psi, double tolerance,
                               double rel_tol, int max_iter, int n_extra, const char *const *keys,
                               const char *const *values, double *out, char *err, int err_len)
{
    return run(solver_name, n, n_faces, diag, lower, upper, lower_addr, upper_addr, source, psi, tolerance,
               rel_tol, max_iter, n_extra, keys, values, Coupling(), out, err, err_len, slot);
}

/* The same with a cyclic patch pair: face f of patch A (cell fcA[f])
 * coupled to face f of patch B (cell fcB[f]) with interfaceBouCoeffs
 * coeffA / coeffB; processor != 0 adds a processor patch. */
int mf_solve_coupled(const char *solver_name, int n, int n_faces, const double *diag, const double *lower,
                     const double *upper, const int *lower_addr, const int *upper_addr,
                     const double *source, double *psi, double tolerance, double rel_tol, int max_iter,
                     int n_extra, const char *const *keys, const char *const *values, int n_cyc,
                     const int *fcA, const int *fcB, const double *coeffA, const double *coeffB,
                     int processor, double *out, char *err, int err_len)
{
    Coupling c;
    c.n_cyc = n_cyc;
    c.fcA = fcA;
    c.fcB = fcB;
    c.coeffA = coeffA;
    c.coeffB = coeffB;
    c.processor = processor != 0;
    return run(solver_name, n, n_faces, diag, lower, upper, lower_addr, upper_addr, source, psi, tolerance,
               rel_tol, max_iter, n_extra, keys, values, c, out, err, err_len);
}

/* mf_solve_coupled on the lduAddressing object of `slot` (0..3), kept
 * between calls (see mf_solve_reused_addressing). */
int mf_solve_coupled_reused(int slot, const char *solver_name, int n, int n_faces, const double *diag,
                            const double *lower, const double *upper, const int *lower_addr,
                            const int *upper_addr, const double *source, double *psi, double tolerance,
                            double rel_tol, int max_iter, int n_extra, const char *const *keys,
                            const char *const *values, int n_cyc, const int *fcA, const int *fcB,
                            const double *coeffA, const double *coeffB, double *out, char *err, int err_len)
{
    Coupling c;
    c.n_cyc = n_cyc;
    c.fcA = fcA;
    c.fcB = fcB;
    c.coeffA = coeffA;
    c.coeffB = coeffB;
    return run(solver_name, n, n_faces, diag, lower, upper, lower_addr, upper_addr, source, psi, tolerance,
               rel_tol, max_iter, n_extra, keys, values, c, out, err, err_len, slot);
}

/* The parallel run's transport (minifoam's Pstream): NULL ends the
 * parallel run.  The structure must stay valid while it is installed. */
void mf_set_transport(const Foam::mfTransport *t)
{
    Foam::UPstream::transport() = t;
    Foam::UPstream::requests().clear();
}

/* mf_solve on one subdomain of a decomposed case (a parallel run: install
 * the transport first), with n_proc processor patches (see Coupling). */
int mf_solve_decomposed(const char *solver_name, int n, int n_faces, const double *diag, const double *lower,
                        const double *upper, const int *lower_addr, const int *upper_addr,
                        const double *source, double *psi, double tolerance, double rel_tol, int max_iter,
                        int n_extra, const char *const *keys, const char *const *values, int n_proc,
                        const int *proc_neighbour, const int *proc_size, const int *proc_cells,
                        const double *proc_coeffs, double *out, char *err, int err_len)
{
    Coupling c;
    c.n_proc = n_proc;
    c.proc_neighbour = proc_neighbour;
    c.proc_size = proc_size;
    c.proc_cells = proc_cells;
    c.proc_coeffs = proc_coeffs;
    return run(solver_name, n, n_faces, diag, lower, upper, lower_addr, upper_addr, source, psi, tolerance,
               rel_tol, max_iter, n_extra, keys, values, c, out, err, err_len);
}

/* The plugin's processor-patch callbacks (cuFoamGB300Comm.H) without a
 * solve: the interfaces of n_proc patches as in mf_solve_decomposed, one
 * exchange of send[] (the values of the face cells, patch after patch)
 * into recv[], then a sum over the ranks of values[0..n_values) and a
 * maximum of max_values[0..n_values).  Returns 0, 1 when a callback
 * failed, -1 on a FatalError (text in err). */
int mf_processor_comm_check(int n_proc, const int *proc_neighbour, const int *proc_size, const int *proc_cells,
                            const double *proc_coeffs, const double *send, double *recv, int count,
                            double *values, double *max_values, int n_values, char *err, int err_len)
{
    try {
        using namespace Foam;
        Coupling c;
        c.n_proc = n_proc;
        c.proc_neighbour = proc_neighbour;
        c.proc_size = proc_size;
        c.proc_cells = proc_cells;
        c.proc_coeffs = proc_coeffs;
        FieldField<Field, scalar> bou, intc;
        lduInterfaceFieldPtrsList interfaces;
        bou.resize(1);
        intc.resize(1);
        interfaces.push_back(nullptr);
        ProcessorPatches procs;
        procs.add(c, bou, intc, interfaces);
        const cuFoamGB300ProcessorComm comm(interfaces, bou);
        const cf_interfaces ifc = comm.interfaces();
        const cf_comm cc = comm.comm();
        for (int f = 0; f < ifc.n_faces; ++f)
            if (ifc.face_cells[f] != proc_cells[f] || ifc.coeffs[f] != proc_coeffs[f]) return 2;
        if (cc.exchange(cc.user, send, recv, count) != 0) return 1;
        if (cc.allreduce_sum(cc.user, values, n_values) != 0) return 1;
        if (cc.allreduce_max(cc.user, max_values, n_values) != 0) return 1;
        if (err && err_len > 0) err[0] = 0;
        return 0;
    } catch (const std::exception &e) {
        if (err && err_len > 0) {
            std::strncpy(err, e.what(), err_len - 1);
            err[err_len - 1] = 0;
        }
        return -1;
    }
}

} // extern "C"
