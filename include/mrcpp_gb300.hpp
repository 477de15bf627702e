// mrcpp_gb300.hpp -- header-only mrcpp:: shim over the C ABI (mw_gb300.h).
//
// Gives MRChem's hot-path call sites the same spelling they use with MRCPP
// (commit 0e5b32003eed8e1abb22a44ba4e1a2ce9fd9ddb1):
//   MultiResolutionAnalysis<3>(BoundingBox<3>(...), InterpolatingBasis(k), depth)  src/mrenv.cpp:105-122
//   FunctionTree<3>(MRA)                                        src/qmfunctions/density_utils.cpp:71
//   PoissonOperator(MRA, prec)                                  src/driver.cpp:1131,1283
//   HelmholtzOperator(MRA, mu, prec)                            src/scf_solver/HelmholtzVector.cpp:144
//   apply(prec, out, oper, inp[, precTrees], maxIter, absPrec)  CoulombPotential.cpp:131, HelmholtzVector.cpp:149
//   multiply / square / add / build_grid / copy_grid / copy_func / clear
//                                                               QMPotential.cpp:146-147, density_utils.cpp:72-87
// A non-zero status from the engine becomes an mrcpp::Error exception, the
// counterpart of MRCPP's MSG_ERROR / MSG_ABORT (the engine never aborts).
#pragma once

#include <array>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "mw_gb300.h"

namespace mrcpp {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc, mw_ctx ctx) {
    if (rc != MW_OK) throw Error(rc, std::string("mrchem_gb300: ") + mw_last_error(ctx));
}

template <int D> class BoundingBox;
template <> class BoundingBox<3> {
public:
    BoundingBox(int scale, const std::array<int, 3> &corner, const std::array<int, 3> &boxes)
            : scale_(scale), corner_(corner), boxes_(boxes) {}
    BoundingBox(int scale, const std::array<int, 3> &corner, const std::array<int, 3> &boxes,
                const std::array<double, 3> &sfac)
            : BoundingBox(scale, corner, boxes) {
        for (double s : sfac)
            if (s != 1.0) throw Error(MW_ERR_ARG, "scaling factors other than 1 are not supported");
    }
    int scale_;
    std::array<int, 3> corner_, boxes_;
};

struct InterpolatingBasis {
    explicit InterpolatingBasis(int k) : order(k) {}
    int order;
    static constexpr int type = MW_BASIS_INTERPOLATING;
};
struct LegendreBasis {
    explicit LegendreBasis(int k) : order(k) {}
    int order;
    static constexpr int type = MW_BASIS_LEGENDRE;
};

template <int D> class MultiResolutionAnalysis;
template <> class MultiResolutionAnalysis<3> {
public:
    template <class Basis>
    MultiResolutionAnalysis(const BoundingBox<3> &box, const Basis &basis, int max_depth, int device = 0) {
        check(mw_ctx_create(device, box.scale_, box.corner_.data(), box.boxes_.data(), basis.order, Basis::type,
                            max_depth, &ctx_),
              nullptr);
    }
    ~MultiResolutionAnalysis() { mw_ctx_destroy(ctx_); }
    MultiResolutionAnalysis(const MultiResolutionAnalysis &) = delete;
    MultiResolutionAnalysis &operator=(const MultiResolutionAnalysis &) = delete;
    mw_ctx handle() const { return ctx_; }

private:
    mw_ctx ctx_ = nullptr;
};

template <int D> class FunctionTree;
template <> class FunctionTree<3> {
public:
    explicit FunctionTree(const MultiResolutionAnalysis<3> &mra) : ctx_(mra.handle()) {
        check(mw_tree_create(ctx_, &t_), ctx_);
    }
    ~FunctionTree() { mw_tree_destroy(t_); }
    FunctionTree(const FunctionTree &) = delete;
    FunctionTree &operator=(const FunctionTree &) = delete;
    int getNNodes() const {
        int n = 0;
        check(mw_tree_nnodes(t_, &n), ctx_);
        return n;
    }
    double getSquareNorm() const {
        double v = 0;
        check(mw_tree_squared_norm(t_, &v), ctx_);
        return v;
    }
    double integrate() const {
        double v = 0;
        check(mw_tree_integrate(t_, &v), ctx_);
        return v;
    }
    void rescale(double c) { check(mw_tree_rescale(t_, c), ctx_); }
    void crop(double prec, bool absPrec = false) { check(mw_crop(t_, prec, absPrec ? 1 : 0), ctx_); }
    void clear() { check(mw_tree_clear(t_), ctx_); }
    mw_tree handle() const { return t_; }
    mw_ctx context() const { return ctx_; }

private:
    mw_ctx ctx_;
    mw_tree t_ = nullptr;
};

template <int D> using FunctionTreeVector = std::vector<std::tuple<double, FunctionTree<D> *>>;

class ConvolutionOperatorBase {
public:
    ~ConvolutionOperatorBase() {
        if (op_) mw_op_destroy(op_);
    }
    mw_op handle() const { return op_; }

protected:
    mw_op op_ = nullptr;
};

class PoissonOperator : public ConvolutionOperatorBase {
public:
    PoissonOperator(const MultiResolutionAnalysis<3> &mra, double prec) {
        check(mw_op_create_poisson(mra.handle(), prec, &op_), mra.handle());
    }
};

class HelmholtzOperator : public ConvolutionOperatorBase {
public:
    HelmholtzOperator(const MultiResolutionAnalysis<3> &mra, double mu, double prec) {
        check(mw_op_create_helmholtz(mra.handle(), mu, prec, &op_), mra.handle());
    }
};

// precision policy for the shim's apply (the reference computes in FP64 only)
inline int &apply_precision_mode() {
    static int mode = MW_PREC_FP64;
    return mode;
}

template <int D>
void apply(double prec, FunctionTree<D> &out, ConvolutionOperatorBase &oper, FunctionTree<D> &inp, int maxIter = -1,
           bool absPrec = false) {
    check(mw_apply(prec, out.handle(), oper.handle(), inp.handle(), 0, nullptr, maxIter, absPrec ? 1 : 0,
                   apply_precision_mode()),
          out.context());
}

template <int D>
void apply(double prec, FunctionTree<D> &out, ConvolutionOperatorBase &oper, FunctionTree<D> &inp,
           FunctionTreeVector<D> &precTrees, int maxIter = -1, bool absPrec = false) {
    std::vector<mw_tree> pt;
    for (auto &e : precTrees) pt.push_back(std::get<1>(e)->handle());
    check(mw_apply(prec, out.handle(), oper.handle(), inp.handle(), (int)pt.size(), pt.data(), maxIter,
                   absPrec ? 1 : 0, apply_precision_mode()),
          out.context());
}

template <int D>
void multiply(double prec, FunctionTree<D> &out, double coef, FunctionTree<D> &a, FunctionTree<D> &b,
              int maxIter = -1, bool absPrec = false, bool useMaxNorms = false) {
    check(mw_multiply(prec, out.handle(), coef, a.handle(), b.handle(), maxIter, absPrec ? 1 : 0, useMaxNorms ? 1 : 0),
          out.context());
}

template <int D>
void square(double prec, FunctionTree<D> &out, FunctionTree<D> &inp, int maxIter = -1, bool absPrec = false) {
    check(mw_square(prec, out.handle(), inp.handle(), maxIter, absPrec ? 1 : 0), out.context());
}

template <int D>
void add(double prec, FunctionTree<D> &out, FunctionTreeVector<D> &inp, int maxIter = -1) {
    std::vector<double> c;
    std::vector<mw_tree> t;
    for (auto &e : inp) {
        c.push_back(std::get<0>(e));
        t.push_back(std::get<1>(e)->handle());
    }
    check(mw_add(prec, out.handle(), (int)t.size(), c.data(), t.data(), maxIter), out.context());
}

template <int D> void build_grid(FunctionTree<D> &out, FunctionTreeVector<D> &inp) {
    std::vector<mw_tree> t;
    for (auto &e : inp) t.push_back(std::get<1>(e)->handle());
    check(mw_build_grid(out.handle(), (int)t.size(), t.data()), out.context());
}

template <int D> void build_grid(FunctionTree<D> &out, FunctionTree<D> &inp) {
    mw_tree t = inp.handle();
    check(mw_build_grid(out.handle(), 1, &t), out.context());
}

template <int D> void copy_grid(FunctionTree<D> &out, FunctionTree<D> &inp) {
    check(mw_copy_grid(out.handle(), inp.handle()), out.context());
}

template <int D> void copy_func(FunctionTree<D> &out, FunctionTree<D> &inp) {
    check(mw_copy_func(out.handle(), inp.handle()), out.context());
}

template <int D> void clear(FunctionTreeVector<D> &vec, bool dealloc = false) {
    for (auto &e : vec) {
        if (dealloc)
            delete std::get<1>(e);
        else
            std::get<1>(e)->clear();
    }
    vec.clear();
}

template <int D> double dot(FunctionTree<D> &a, FunctionTree<D> &b) {
    double v = 0;
    check(mw_dot(a.handle(), b.handle(), &v), a.context());
    return v;
}

}  // namespace mrcpp
