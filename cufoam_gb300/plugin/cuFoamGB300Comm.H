/*
 * cuFoamGB300Comm.H -- the processor patches of a decomposed case handed to
 * cf_solve_decomposed (include/cufoam_gb300.h), with OpenFOAM's own
 * parallel communication behind its callbacks.
 *
 * In a parallel OpenFOAM run, lduMatrix::Amul finishes every rank's product
 * through the processor interfaces: each sends the values of its face cells
 * to the neighbouring rank (processorLduInterface::send), receives the
 * neighbour's values of the cells across the same faces (receive), and
 * subtracts interfaceBouCoeffs[f] * received[f] from row faceCells[f]
 * (processorFvPatchField::updateInterfaceMatrix); every inner product is
 * reduce(..., sumOp<scalar>()), as gSumProd does.  The library does the
 * arithmetic on the device; the two callbacks below are the transfers:
 *   exchange:      send + receive on every processor interface (non-blocking,
 *                  then Pstream::waitRequests()), the faces patch after patch
 *   allreduce_sum: reduce(value, sumOp<scalar>()) per value -- OpenFOAM's
 *                  own solvers decide convergence on such sums on every rank,
 *                  so they are the same on every rank
 *   allreduce_max: reduce(value, maxOp<scalar>()) (Richardson's power
 *                  method: the smallest |a_ii| of the whole mesh)
 * Compiles against OpenFOAM or the minifoam stand-in.
 */
#ifndef CUFOAM_GB300_COMM_H
#define CUFOAM_GB300_COMM_H

#include "lduMatrix.H"
#include "processorLduInterface.H"
#include "Pstream.H"
#include "PstreamReduceOps.H"
#include "cufoam_gb300.h"

#include <cstdint>
#include <exception>
#include <vector>

namespace Foam {

class cuFoamGB300ProcessorComm {
    struct Patch {
        const processorLduInterface *ifc;
        label offset, size;
    };
    std::vector<Patch> patches_;
    std::vector<int32_t> faceCells_;
    std::vector<double> coeffs_;

    static int32_t exchange(void *user, const double *send, double *recv, int32_t count)
    {
        try {
            const cuFoamGB300ProcessorComm &c = *static_cast<const cuFoamGB300ProcessorComm *>(user);
            if (count != (int32_t)c.faceCells_.size()) return 1;
            for (const Patch &p : c.patches_) {
                const UList<scalar> s(const_cast<scalar *>(send + p.offset), p.size);
                p.ifc->send(Pstream::commsTypes::nonBlocking, s);
            }
            for (const Patch &p : c.patches_) {
                UList<scalar> r(recv + p.offset, p.size);
                p.ifc->receive(Pstream::commsTypes::nonBlocking, r);
            }
            Pstream::waitRequests();
            return 0;
        } catch (const std::exception &) {
            return 1;
        }
    }

    static int32_t allreduceSum(void *, double *values, int32_t count)
    {
        try {
            for (int32_t i = 0; i < count; ++i) reduce(values[i], sumOp<scalar>());
            return 0;
        } catch (const std::exception &) {
            return 1;
        }
    }

    static int32_t allreduceMax(void *, double *values, int32_t count)
    {
        try {
            for (int32_t i = 0; i < count; ++i) reduce(values[i], maxOp<scalar>());
            return 0;
        } catch (const std::exception &) {
            return 1;
        }
    }

public:
    // The processor interfaces of `interfaces`, in patch order, with their
    // interfaceBouCoeffs; other (and unset) patches are skipped.
    cuFoamGB300ProcessorComm(const lduInterfaceFieldPtrsList &interfaces,
                             const FieldField<Field, scalar> &bouCoeffs)
    {
        for (label patchi = 0; patchi < interfaces.size(); ++patchi) {
            if (!interfaces.set(patchi)) continue;
            const lduInterface &ifc = interfaces[patchi].interface();
            if (!isA<processorLduInterface>(ifc)) continue;
            const processorLduInterface &proc = refCast<const processorLduInterface>(ifc);
            const labelList &fc = ifc.faceCells();
            const scalarField &co = bouCoeffs[patchi];
            if (co.size() != fc.size()) {
                FatalErrorInFunction << "cuFoamGB300: processor patch " << patchi
                                     << " has " << co.size() << " coefficients for " << fc.size()
                                     << " faces" << exit(FatalError);
            }
            patches_.push_back(Patch{&proc, (label)faceCells_.size(), fc.size()});
            for (label f = 0; f < fc.size(); ++f) {
                faceCells_.push_back(fc[f]);
                coeffs_.push_back(co[f]);
            }
        }
    }

    label nPatches() const { return (label)patches_.size(); }

    cf_interfaces interfaces() const
    {
        cf_interfaces i;
        i.n_faces = (int32_t)faceCells_.size();
        i.face_cells = faceCells_.data();
        i.coeffs = coeffs_.data();
        return i;
    }

    // the callbacks; valid while this object lives
    cf_comm comm() const
    {
        cf_comm c;
        c.user = const_cast<cuFoamGB300ProcessorComm *>(this);
        c.exchange = &exchange;
        c.allreduce_sum = &allreduceSum;
        c.allreduce_max = &allreduceMax;
        return c;
    }
};

} // namespace Foam

#endif
