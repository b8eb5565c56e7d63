/*
 * minifoam/lduMatrix.H -- a minimal stand-in for the parts of OpenFOAM's API
 * that the cuFoam plugins use (lduMatrix, lduAddressing, lduMatrix::solver
 * with its run-time selection tables, solverPerformance, dictionary, Field,
 * TypeName / defineTypeNameAndDebug, FatalError).  It lets the plugin
 * sources (cuFoamGB300.{H,C}) compile and run without OpenFOAM, in the
 * tests and on machines without an OpenFOAM installation.  Semantics follow
 * OpenFOAM where the plugins depend on them: solver controls tolerance
 * (default 1e-6), relTol (0), maxIter (1000), minIter (0); lower() of a
 * symmetric matrix is upper(); solver selection by name from the symmetric
 * or the asymmetric table; FatalError aborts the call (here: an exception).
 */
#ifndef MINIFOAM_LDUMATRIX_H
#define MINIFOAM_LDUMATRIX_H

#include <cstdint>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace Foam {

typedef int32_t label;
typedef double scalar;
typedef unsigned char direction;

class word : public std::string {
public:
    word() {}
    word(const char *s) : std::string(s) {}
    word(const std::string &s) : std::string(s) {}
};

template <class T>
class List : public std::vector<T> {
public:
    using std::vector<T>::vector;
    const T *cdata() const { return std::vector<T>::data(); }
    T *data() { return std::vector<T>::data(); }
    label size() const { return (label)std::vector<T>::size(); }
};

typedef List<label> labelList;

// a view of contiguous storage (OpenFOAM's UList; List is one here only
// by conversion)
template <class T>
class UList {
    T *v_;
    label size_;

public:
    UList(T *v, label size) : v_(v), size_(size) {}
    label size() const { return size_; }
    T *data() { return v_; }
    const T *cdata() const { return v_; }
    T &operator[](label i) { return v_[i]; }
    const T &operator[](label i) const { return v_[i]; }
};

// ---- the parallel run (OpenFOAM's UPstream / Pstream) ---------------------
// The stand-in moves no data itself: a harness that emulates a parallel run
// installs a transport, which completes the posted non-blocking sends and
// receives together (waitRequests) and sums reductions over the ranks.
// Without a transport the run is serial (parRun() false).
struct mfTransport {
    int32_t myProcNo, nProcs;
    void *user;
    // kind[i]: 0 send, 1 receive; the rest as MPI_Isend / MPI_Irecv
    int32_t (*complete)(void *user, int32_t n, const int32_t *kind, const int32_t *peer,
                        const int32_t *tag, void *const *data, const int64_t *bytes);
    int32_t (*allreduceSum)(void *user, double *values, int32_t count);
    int32_t (*allreduceMax)(void *user, double *values, int32_t count);
};

class UPstream {
public:
    enum class commsTypes { blocking, scheduled, nonBlocking };

    struct Request {
        int32_t kind, peer, tag;
        void *data;
        int64_t bytes;
    };

    static const mfTransport *&transport()
    {
        static const mfTransport *t = nullptr;
        return t;
    }
    static std::vector<Request> &requests()
    {
        static std::vector<Request> r;
        return r;
    }
    static bool parRun() { return transport() != nullptr; }
    static int myProcNo() { return parRun() ? transport()->myProcNo : 0; }
    static int nProcs() { return parRun() ? transport()->nProcs : 1; }
    static void post(int32_t kind, int32_t peer, int32_t tag, void *data, int64_t bytes)
    {
        if (!parRun()) throw std::runtime_error("Pstream: communication in a serial run");
        requests().push_back(Request{kind, peer, tag, data, bytes});
    }
    static void waitRequests()
    {
        std::vector<Request> &r = requests();
        if (r.empty()) return;
        std::vector<int32_t> kind, peer, tag;
        std::vector<void *> data;
        std::vector<int64_t> bytes;
        for (const Request &q : r) {
            kind.push_back(q.kind);
            peer.push_back(q.peer);
            tag.push_back(q.tag);
            data.push_back(q.data);
            bytes.push_back(q.bytes);
        }
        r.clear();
        const mfTransport *t = transport();
        if (t->complete(t->user, (int32_t)kind.size(), kind.data(), peer.data(), tag.data(), data.data(),
                        bytes.data()) != 0)
            throw std::runtime_error("Pstream: a transfer failed");
    }
};

class Pstream : public UPstream {};

template <class T>
struct sumOp {
    T operator()(const T &a, const T &b) const { return a + b; }
};

template <class T>
struct maxOp {
    T operator()(const T &a, const T &b) const { return a > b ? a : b; }
};

// reduce(value, sumOp<scalar>()) / reduce(value, maxOp<scalar>()): the sum
// or the maximum over all ranks, on every rank
inline void reduce(double &v, const sumOp<double> &)
{
    if (!UPstream::parRun()) return;
    const mfTransport *t = UPstream::transport();
    if (t->allreduceSum(t->user, &v, 1) != 0) throw std::runtime_error("Pstream: a reduction failed");
}
inline void reduce(double &v, const maxOp<double> &)
{
    if (!UPstream::parRun()) return;
    const mfTransport *t = UPstream::transport();
    if (t->allreduceMax(t->user, &v, 1) != 0) throw std::runtime_error("Pstream: a reduction failed");
}

template <class T>
class Field : public List<T> {
public:
    using List<T>::List;
};

typedef Field<scalar> scalarField;

template <template <class> class F, class T>
class FieldField : public std::vector<F<T>> {};

// ---- coupled interfaces (OpenFOAM's lduInterface / lduInterfaceField) -----
class lduInterface {
public:
    virtual ~lduInterface() {}
    virtual const labelList &faceCells() const = 0;
};

// a cyclic patch couples its face cells to the face cells of its
// neighbour patch (cyclicLduInterface::neighbPatch)
class cyclicLduInterface : public lduInterface {
    labelList faceCells_;
    const cyclicLduInterface *nbr_ = nullptr;

public:
    explicit cyclicLduInterface(const labelList &faceCells) : faceCells_(faceCells) {}
    void setNeighbPatch(const cyclicLduInterface &n) { nbr_ = &n; }
    const labelList &faceCells() const override { return faceCells_; }
    const cyclicLduInterface &neighbPatch() const { return *nbr_; }
};

// a processor patch couples to cells of another MPI rank; its faces are
// listed alike on both sides.  send / receive as OpenFOAM's
// processorLduInterface (non-blocking only in the stand-in: completed by
// UPstream::waitRequests()).
class processorLduInterface : public lduInterface {
    labelList faceCells_;
    int neighbProcNo_;
    int tag_;

public:
    explicit processorLduInterface(const labelList &faceCells, int neighbProcNo = -1, int tag = 1)
        : faceCells_(faceCells), neighbProcNo_(neighbProcNo), tag_(tag) {}
    const labelList &faceCells() const override { return faceCells_; }
    int myProcNo() const { return UPstream::myProcNo(); }
    int neighbProcNo() const { return neighbProcNo_; }
    int tag() const { return tag_; }
    template <class Type>
    void send(const UPstream::commsTypes commsType, const UList<Type> &f) const
    {
        if (commsType != UPstream::commsTypes::nonBlocking)
            throw std::runtime_error("processorLduInterface: only non-blocking transfers in the stand-in");
        UPstream::post(0, neighbProcNo_, tag_, const_cast<Type *>(f.cdata()), (int64_t)sizeof(Type) * f.size());
    }
    template <class Type>
    void receive(const UPstream::commsTypes commsType, UList<Type> &f) const
    {
        if (commsType != UPstream::commsTypes::nonBlocking)
            throw std::runtime_error("processorLduInterface: only non-blocking transfers in the stand-in");
        UPstream::post(1, neighbProcNo_, tag_, f.data(), (int64_t)sizeof(Type) * f.size());
    }
};

class lduInterfaceField {
    const lduInterface &interface_;

public:
    explicit lduInterfaceField(const lduInterface &i) : interface_(i) {}
    virtual ~lduInterfaceField() {}
    const lduInterface &interface() const { return interface_; }
};

// UPtrList<const lduInterfaceField>: null entries for uncoupled patches
class lduInterfaceFieldPtrsList : public std::vector<const lduInterfaceField *> {
public:
    using std::vector<const lduInterfaceField *>::vector;
    label size() const { return (label)std::vector<const lduInterfaceField *>::size(); }
    bool set(label i) const { return (*this).std::vector<const lduInterfaceField *>::operator[](i) != nullptr; }
    const lduInterfaceField &operator[](label i) const
    {
        return *std::vector<const lduInterfaceField *>::operator[](i);
    }
};

template <class T, class U>
bool isA(const U &u)
{
    return dynamic_cast<const T *>(&u) != nullptr;
}

template <class To, class From>
To &refCast(From &f)
{
    return dynamic_cast<To &>(f);
}

// ---- errors ----------------------------------------------------------------
struct ExitTag {};
struct FatalErrorType {};
extern FatalErrorType FatalError;
inline ExitTag exit(const FatalErrorType &) { return ExitTag(); }

class FatalErrorStream {
    std::ostringstream os_;

public:
    explicit FatalErrorStream(const char *fn) { os_ << fn << ": "; }
    template <class T>
    FatalErrorStream &operator<<(const T &v)
    {
        os_ << v;
        return *this;
    }
    FatalErrorStream &operator<<(ExitTag) { throw std::runtime_error(os_.str()); }
};

#define FatalErrorInFunction ::Foam::FatalErrorStream(__func__)

// ---- dictionary ------------------------------------------------------------
class dictionary {
    std::map<std::string, std::string> entries_;

    static bool parse(const std::string &s, bool *)
    {
        return s == "true" || s == "yes" || s == "on" || s == "1";
    }
    static label parse(const std::string &s, label *) { return (label)std::stol(s); }
    static scalar parse(const std::string &s, scalar *) { return std::stod(s); }
    static word parse(const std::string &s, word *) { return word(s); }

public:
    void set(const std::string &k, const std::string &v) { entries_[k] = v; }
    bool found(const std::string &k) const { return entries_.count(k) != 0; }
    template <class T>
    T lookupOrDefault(const word &k, const T &deflt) const
    {
        auto it = entries_.find(k);
        if (it == entries_.end()) return deflt;
        return parse(it->second, (T *)nullptr);
    }
    word lookup(const word &k) const
    {
        auto it = entries_.find(k);
        if (it == entries_.end()) throw std::runtime_error("keyword " + k + " is undefined");
        return word(it->second);
    }
};

// ---- solverPerformance -------------------------------------------------------
class solverPerformance {
    word solverName_, fieldName_;
    scalar initialResidual_ = 0, finalResidual_ = 0;
    label nIterations_ = 0;
    bool converged_ = false, singular_ = false;

public:
    solverPerformance() {}
    solverPerformance(const word &solverName, const word &fieldName)
        : solverName_(solverName), fieldName_(fieldName) {}
    const word &solverName() const { return solverName_; }
    const word &fieldName() const { return fieldName_; }
    scalar &initialResidual() { return initialResidual_; }
    scalar initialResidual() const { return initialResidual_; }
    scalar &finalResidual() { return finalResidual_; }
    scalar finalResidual() const { return finalResidual_; }
    label &nIterations() { return nIterations_; }
    label nIterations() const { return nIterations_; }
    bool converged() const { return converged_; }
    bool singular() const { return singular_; }
    bool checkConvergence(const scalar tolerance, const scalar relTolerance)
    {
        converged_ = finalResidual_ < tolerance ||
                     (relTolerance > 1e-20 && finalResidual_ < relTolerance * initialResidual_);
        return converged_;
    }
};

// ---- run-time type names -----------------------------------------------------
#define TypeName(TypeNameString)                                          \
    static const char *typeName_() { return TypeNameString; }             \
    static const ::Foam::word typeName;                                   \
    virtual const ::Foam::word &type() const { return typeName; }

#define defineTypeNameAndDebug(Type, DebugSwitch) \
    const ::Foam::word Type::typeName(Type::typeName_())

// ---- addressing and matrix ---------------------------------------------------
class lduAddressing {
    label size_;
    labelList lower_, upper_, losort_, losortStart_, ownerStart_;

public:
    lduAddressing(label nCells, const labelList &lowerAddr, const labelList &upperAddr)
        : size_(nCells), lower_(lowerAddr), upper_(upperAddr)
    {
        calcAddressing();
    }
    // New faces in the same memory (the stand-in's way to model a mesh that
    // reuses an old one's storage: same object, same list buffers when the
    // sizes match, other contents).
    void reset(label nCells, const labelList &lowerAddr, const labelList &upperAddr)
    {
        size_ = nCells;
        lower_.assign(lowerAddr.begin(), lowerAddr.end());
        upper_.assign(upperAddr.begin(), upperAddr.end());
        calcAddressing();
    }
    label size() const { return size_; }
    const labelList &lowerAddr() const { return lower_; }
    const labelList &upperAddr() const { return upper_; }
    const labelList &losortAddr() const { return losort_; }
    const labelList &losortStartAddr() const { return losortStart_; }
    const labelList &ownerStartAddr() const { return ownerStart_; }

private:
    // losort: faces stably sorted by neighbour; starts: first position
    // (first face) whose neighbour (owner) is >= cell
    void calcAddressing()
    {
        const label nf = lower_.size();
        std::vector<label> count(size_ + 1, 0);
        for (label f = 0; f < nf; ++f) ++count[upper_[f] + 1];
        for (label c = 0; c < size_; ++c) count[c + 1] += count[c];
        losortStart_.assign(count.begin(), count.end());
        losort_.assign(nf, -1);
        for (label f = 0; f < nf; ++f) losort_[count[upper_[f]]++] = f;
        ownerStart_.assign(size_ + 1, nf);
        label f = 0;
        for (label c = 0; c <= size_; ++c) {
            while (f < nf && lower_[f] < c) ++f;
            ownerStart_[c] = f;
        }
    }
};

class lduMatrix {
    const lduAddressing &addr_;
    scalarField diag_, lower_, upper_;
    bool hasLower_, hasUpper_;

public:
    // symmetric when lower is not given
    lduMatrix(const lduAddressing &addr, const scalarField &diag, const scalarField *lower,
              const scalarField *upper)
        : addr_(addr), diag_(diag), hasLower_(lower != nullptr), hasUpper_(upper != nullptr)
    {
        if (lower) lower_ = *lower;
        if (upper) upper_ = *upper;
    }
    const lduAddressing &lduAddr() const { return addr_; }
    const scalarField &diag() const { return diag_; }
    const scalarField &upper() const { return hasUpper_ ? upper_ : lower_; }
    const scalarField &lower() const { return hasLower_ ? lower_ : upper_; }
    bool symmetric() const { return hasUpper_ && !hasLower_; }
    bool asymmetric() const { return hasUpper_ && hasLower_; }

    class solver {
    protected:
        word fieldName_;
        const lduMatrix &matrix_;
        const FieldField<Field, scalar> &interfaceBouCoeffs_;
        const FieldField<Field, scalar> &interfaceIntCoeffs_;
        const lduInterfaceFieldPtrsList &interfaces_;
        dictionary controlDict_;
        label maxIter_, minIter_;
        scalar tolerance_, relTol_;

    public:
        typedef solver *(*constructor)(const word &, const lduMatrix &,
                                       const FieldField<Field, scalar> &,
                                       const FieldField<Field, scalar> &,
                                       const lduInterfaceFieldPtrsList &, const dictionary &);
        static std::map<std::string, constructor> &symMatrixConstructorTable()
        {
            static std::map<std::string, constructor> t;
            return t;
        }
        static std::map<std::string, constructor> &asymMatrixConstructorTable()
        {
            static std::map<std::string, constructor> t;
            return t;
        }
        template <class T>
        static solver *make(const word &f, const lduMatrix &m, const FieldField<Field, scalar> &b,
                            const FieldField<Field, scalar> &i, const lduInterfaceFieldPtrsList &in,
                            const dictionary &d)
        {
            return new T(f, m, b, i, in, d);
        }
        template <class T>
        struct addsymMatrixConstructorToTable {
            addsymMatrixConstructorToTable() { symMatrixConstructorTable()[T::typeName] = &make<T>; }
        };
        template <class T>
        struct addasymMatrixConstructorToTable {
            addasymMatrixConstructorToTable() { asymMatrixConstructorTable()[T::typeName] = &make<T>; }
        };

        solver(const word &fieldName, const lduMatrix &matrix,
               const FieldField<Field, scalar> &interfaceBouCoeffs,
               const FieldField<Field, scalar> &interfaceIntCoeffs,
               const lduInterfaceFieldPtrsList &interfaces, const dictionary &solverControls)
            : fieldName_(fieldName), matrix_(matrix), interfaceBouCoeffs_(interfaceBouCoeffs),
              interfaceIntCoeffs_(interfaceIntCoeffs), interfaces_(interfaces), controlDict_(solverControls)
        {
            maxIter_ = controlDict_.lookupOrDefault<label>("maxIter", 1000);
            minIter_ = controlDict_.lookupOrDefault<label>("minIter", 0);
            tolerance_ = controlDict_.lookupOrDefault<scalar>("tolerance", 1e-6);
            relTol_ = controlDict_.lookupOrDefault<scalar>("relTol", 0);
        }
        virtual ~solver() {}
        virtual const word &type() const = 0;
        const word &fieldName() const { return fieldName_; }
        const lduMatrix &matrix() const { return matrix_; }
        const dictionary &controlDict() const { return controlDict_; }
        const FieldField<Field, scalar> &interfaceBouCoeffs() const { return interfaceBouCoeffs_; }
        const FieldField<Field, scalar> &interfaceIntCoeffs() const { return interfaceIntCoeffs_; }
        const lduInterfaceFieldPtrsList &interfaces() const { return interfaces_; }
        virtual solverPerformance solve(scalarField &psi, const scalarField &source,
                                        const direction cmpt = 0) const = 0;

        static std::unique_ptr<solver> New(const word &fieldName, const lduMatrix &matrix,
                                           const FieldField<Field, scalar> &bou,
                                           const FieldField<Field, scalar> &intc,
                                           const lduInterfaceFieldPtrsList &interfaces,
                                           const dictionary &controls)
        {
            const word name = controls.lookup("solver");
            auto &table = matrix.symmetric() ? symMatrixConstructorTable() : asymMatrixConstructorTable();
            auto it = table.find(name);
            if (it == table.end())
                throw std::runtime_error("Unknown " +
                                         std::string(matrix.symmetric() ? "symmetric" : "asymmetric") +
                                         " matrix solver " + name);
            return std::unique_ptr<solver>(it->second(fieldName, matrix, bou, intc, interfaces, controls));
        }
    };
};

} // namespace Foam

#endif
