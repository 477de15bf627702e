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
//   project(prec, tree, GaussExp<3>)                            density / initial-guess projections
//   ComplexFunction (alloc/free/add/crop/rescale/norm/squaredNorm/dagger/getNNodes)
//                                                               src/qmfunctions/Orbital.h:51
//   cplxfunc::multiply / multiply_real / multiply_imag          ExchangePotential.cpp:175, density_utils.cpp:180,208
//   cplxfunc::linear_combination                                src/scf_solver/KAIN.cpp:170,182
//   cplxfunc::project, cplxfunc::dot                            exchange_operator.cpp / orbital::dot
// A non-zero status from the engine becomes an mrcpp::Error exception, the
// counterpart of MRCPP's MSG_ERROR / MSG_ABORT (the engine never aborts).
//
// Precision policy: the reference computes in FP64 only.  Each operator carries its
// own mode (ConvolutionOperatorBase::setPrecision, MW_PREC_FP64 by default), so one
// caller can apply a Helmholtz operator in MW_PREC_MIXED while another applies a
// Poisson operator in FP64, from different threads, without shared state.
#pragma once

#include <array>
#include <cmath>
#include <complex>
#include <memory>
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
    ConvolutionOperatorBase() = default;
    ConvolutionOperatorBase(const ConvolutionOperatorBase &) = delete;
    ConvolutionOperatorBase &operator=(const ConvolutionOperatorBase &) = delete;
    ~ConvolutionOperatorBase() {
        if (op_) mw_op_destroy(op_);
    }
    mw_op handle() const { return op_; }
    // arithmetic of this operator's applies: MW_PREC_FP64 (default, the reference's), MW_PREC_MIXED, ...
    void setPrecision(int mode) { mode_ = mode; }
    int getPrecision() const { return mode_; }

protected:
    mw_op op_ = nullptr;
    int mode_ = MW_PREC_FP64;
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

template <int D>
void apply(double prec, FunctionTree<D> &out, ConvolutionOperatorBase &oper, FunctionTree<D> &inp, int maxIter = -1,
           bool absPrec = false) {
    check(mw_apply(prec, out.handle(), oper.handle(), inp.handle(), 0, nullptr, maxIter, absPrec ? 1 : 0,
                   oper.getPrecision()),
          out.context());
}

template <int D>
void apply(double prec, FunctionTree<D> &out, ConvolutionOperatorBase &oper, FunctionTree<D> &inp,
           FunctionTreeVector<D> &precTrees, int maxIter = -1, bool absPrec = false) {
    std::vector<mw_tree> pt;
    for (auto &e : precTrees) pt.push_back(std::get<1>(e)->handle());
    check(mw_apply(prec, out.handle(), oper.handle(), inp.handle(), (int)pt.size(), pt.data(), maxIter,
                   absPrec ? 1 : 0, oper.getPrecision()),
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

// ---- Gaussian expansions and projection ------------------------------------------------------

// c * (x-X)^px (y-Y)^py (z-Z)^pz * exp(-alpha |r-R|^2)
template <int D> class GaussFunc;
template <> class GaussFunc<3> {
public:
    GaussFunc(double alpha, double coef, const std::array<double, 3> &pos = {0.0, 0.0, 0.0},
              const std::array<int, 3> &power = {0, 0, 0})
            : alpha_(alpha), coef_(coef), pos_(pos), power_(power) {}
    double alpha_, coef_;
    std::array<double, 3> pos_;
    std::array<int, 3> power_;
};

template <int D> class GaussExp;
template <> class GaussExp<3> {
public:
    void append(const GaussFunc<3> &g) { terms_.push_back(g); }
    int size() const { return (int)terms_.size(); }
    const GaussFunc<3> &getFunc(int i) const { return terms_.at(i); }

private:
    std::vector<GaussFunc<3>> terms_;
};

// mrcpp::project(prec, out, GaussExp<3>&, maxIter, absPrec): adaptive projection of a Gaussian sum
inline void project(double prec, FunctionTree<3> &out, const GaussExp<3> &inp, int maxIter = -1, bool absPrec = false) {
    (void)maxIter;
    std::vector<mw_gterm> t(inp.size());
    for (int i = 0; i < inp.size(); i++) {
        const GaussFunc<3> &g = inp.getFunc(i);
        t[i].coef = g.coef_;
        t[i].alpha = g.alpha_;
        for (int d = 0; d < 3; d++) {
            t[i].pos[d] = g.pos_[d];
            t[i].pw[d] = g.power_[d];
        }
        t[i].pad = 0;
    }
    check(mw_project_gauss(prec, out.handle(), (int)t.size(), t.data(), absPrec ? 1 : 0), out.context());
}

// ---- complex functions (mrcpp::ComplexFunction, the type of MRChem's orbitals, Orbital.h:51) -----

enum class NUMBER { Total, Real, Imag };

using ComplexDouble = std::complex<double>;

// Real and imaginary parts as two optional trees, shared between copies (a copy is a handle, as
// in MRCPP).  dagger() returns a handle to the same trees with the conjugation flag flipped: the
// function it represents is real - i imag.
class ComplexFunction {
public:
    explicit ComplexFunction(const MultiResolutionAnalysis<3> &mra) : mra_(&mra), d_(std::make_shared<Data>()) {}

    ComplexFunction paramCopy() const { return ComplexFunction(*mra_); }
    ComplexFunction dagger() const {
        ComplexFunction out(*this);
        out.conj_ = !conj_;
        return out;
    }
    bool conjugate() const { return conj_; }
    bool hasReal() const { return (bool)d_->re; }
    bool hasImag() const { return (bool)d_->im; }
    FunctionTree<3> &real() const {
        if (!d_->re) throw Error(MW_ERR_STATE, "ComplexFunction: no real part");
        return *d_->re;
    }
    FunctionTree<3> &imag() const {
        if (!d_->im) throw Error(MW_ERR_STATE, "ComplexFunction: no imaginary part");
        return *d_->im;
    }
    const MultiResolutionAnalysis<3> &mra() const { return *mra_; }

    void alloc(NUMBER type) {
        if ((type == NUMBER::Real || type == NUMBER::Total) && !d_->re) d_->re.reset(new FunctionTree<3>(*mra_));
        if ((type == NUMBER::Imag || type == NUMBER::Total) && !d_->im) d_->im.reset(new FunctionTree<3>(*mra_));
    }
    void free(NUMBER type) {
        if (type == NUMBER::Real || type == NUMBER::Total) d_->re.reset();
        if (type == NUMBER::Imag || type == NUMBER::Total) d_->im.reset();
    }
    int getNNodes(NUMBER type) const {
        int n = 0;
        if ((type == NUMBER::Real || type == NUMBER::Total) && hasReal()) n += real().getNNodes();
        if ((type == NUMBER::Imag || type == NUMBER::Total) && hasImag()) n += imag().getNNodes();
        return n;
    }
    double squaredNorm() const {
        double v = 0.0;
        if (hasReal()) v += real().getSquareNorm();
        if (hasImag()) v += imag().getSquareNorm();
        return v;
    }
    double norm() const { return std::sqrt(squaredNorm()); }
    void crop(double prec) {
        if (hasReal()) real().crop(prec);
        if (hasImag()) imag().crop(prec);
    }
    // this <- c * this
    void rescale(double c) {
        if (hasReal()) real().rescale(c);
        if (hasImag()) imag().rescale(c);
    }
    void rescale(ComplexDouble c);
    // this <- this + c * inp on the union grid (ComplexFunction::add)
    void add(ComplexDouble c, const ComplexFunction &inp);

    // the stored parts with their signs in the represented function: f = re + i (sgn_im) im
    double imagSign() const { return conj_ ? -1.0 : 1.0; }

private:
    struct Data {
        std::unique_ptr<FunctionTree<3>> re, im;
    };
    const MultiResolutionAnalysis<3> *mra_;
    std::shared_ptr<Data> d_;
    bool conj_ = false;
    friend void replace_part(ComplexFunction &f, NUMBER part, std::unique_ptr<FunctionTree<3>> t);
};

inline void replace_part(ComplexFunction &f, NUMBER part, std::unique_ptr<FunctionTree<3>> t) {
    if (part == NUMBER::Real)
        f.d_->re = std::move(t);
    else
        f.d_->im = std::move(t);
}

namespace detail {
// out <- sum_i c_i t_i on the trees' union grid; terms with a zero coefficient are left out
inline std::unique_ptr<FunctionTree<3>> combine(const MultiResolutionAnalysis<3> &mra, double prec,
                                                const std::vector<std::tuple<double, FunctionTree<3> *>> &terms) {
    std::vector<double> c;
    std::vector<mw_tree> t;
    for (auto &e : terms)
        if (std::get<0>(e) != 0.0 && std::get<1>(e)) {
            c.push_back(std::get<0>(e));
            t.push_back(std::get<1>(e)->handle());
        }
    if (t.empty()) return nullptr;
    std::unique_ptr<FunctionTree<3>> out(new FunctionTree<3>(mra));
    check(mw_add(prec, out->handle(), (int)t.size(), c.data(), t.data(), -1), out->context());
    return out;
}
}  // namespace detail

inline void ComplexFunction::add(ComplexDouble c, const ComplexFunction &inp) {
    // (re + i s im) + (cr + i ci)(x + i t y) = (re + cr x - ci t y) + i (s im + ci x + cr t y)
    const double s = imagSign(), t = inp.imagSign();
    FunctionTree<3> *x = inp.hasReal() ? &inp.real() : nullptr, *y = inp.hasImag() ? &inp.imag() : nullptr;
    auto re = detail::combine(*mra_, -1.0, {std::make_tuple(1.0, hasReal() ? &real() : nullptr),
                                            std::make_tuple(c.real(), x), std::make_tuple(-c.imag() * t, y)});
    // the stored imaginary part keeps this function's conjugation flag: im' = s * (new imaginary part)
    auto im = detail::combine(*mra_, -1.0, {std::make_tuple(1.0, hasImag() ? &imag() : nullptr),
                                            std::make_tuple(s * c.imag(), x), std::make_tuple(s * c.real() * t, y)});
    if (re) replace_part(*this, NUMBER::Real, std::move(re));
    if (im) replace_part(*this, NUMBER::Imag, std::move(im));
}

inline void ComplexFunction::rescale(ComplexDouble c) {
    if (c.imag() == 0.0) return rescale(c.real());
    // c (re + i s im) = (cr re - ci s im) + i (ci re + cr s im); the stored imaginary part is s times it
    const double s = imagSign();
    FunctionTree<3> *x = hasReal() ? &real() : nullptr, *y = hasImag() ? &imag() : nullptr;
    auto re = detail::combine(*mra_, -1.0, {std::make_tuple(c.real(), x), std::make_tuple(-c.imag() * s, y)});
    auto im = detail::combine(*mra_, -1.0, {std::make_tuple(s * c.imag(), x), std::make_tuple(c.real(), y)});
    replace_part(*this, NUMBER::Real, std::move(re));
    replace_part(*this, NUMBER::Imag, std::move(im));
}

namespace cplxfunc {

// one product of real trees into a new tree: adaptive (prec > 0) or on the union grid (prec < 0)
inline std::unique_ptr<FunctionTree<3>> product(const MultiResolutionAnalysis<3> &mra, double prec, double coef,
                                                FunctionTree<3> &a, FunctionTree<3> &b, bool absPrec,
                                                bool useMaxNorms) {
    std::unique_ptr<FunctionTree<3>> t(new FunctionTree<3>(mra));
    if (prec < 0.0) {
        mw_tree ab[2] = {a.handle(), b.handle()};
        check(mw_build_grid(t->handle(), 2, ab), t->context());
        check(mw_multiply(1.0, t->handle(), coef, a.handle(), b.handle(), 0, 0, 0), t->context());
    } else {
        check(mw_multiply(prec, t->handle(), coef, a.handle(), b.handle(), -1, absPrec ? 1 : 0, useMaxNorms ? 1 : 0),
              t->context());
    }
    return t;
}

// out = Re(a * b), with a's and b's conjugation flags (mrcpp::cplxfunc::multiply_real)
inline void multiply_real(ComplexFunction &out, const ComplexFunction &a, const ComplexFunction &b, double prec,
                          bool absPrec = false, bool useMaxNorms = false) {
    const auto &mra = a.mra();
    std::unique_ptr<FunctionTree<3>> rr, ii;
    if (a.hasReal() && b.hasReal()) rr = product(mra, prec, 1.0, a.real(), b.real(), absPrec, useMaxNorms);
    if (a.hasImag() && b.hasImag())
        ii = product(mra, prec, -1.0 * a.imagSign() * b.imagSign(), a.imag(), b.imag(), absPrec, useMaxNorms);
    if (rr && ii)
        replace_part(out, NUMBER::Real,
                     detail::combine(mra, prec, {std::make_tuple(1.0, rr.get()), std::make_tuple(1.0, ii.get())}));
    else if (rr || ii)
        replace_part(out, NUMBER::Real, rr ? std::move(rr) : std::move(ii));
}

// out = Im(a * b) (mrcpp::cplxfunc::multiply_imag); out is not conjugated
inline void multiply_imag(ComplexFunction &out, const ComplexFunction &a, const ComplexFunction &b, double prec,
                          bool absPrec = false, bool useMaxNorms = false) {
    const auto &mra = a.mra();
    std::unique_ptr<FunctionTree<3>> ri, ir;
    if (a.hasReal() && b.hasImag()) ri = product(mra, prec, b.imagSign(), a.real(), b.imag(), absPrec, useMaxNorms);
    if (a.hasImag() && b.hasReal()) ir = product(mra, prec, a.imagSign(), a.imag(), b.real(), absPrec, useMaxNorms);
    if (ri && ir)
        replace_part(out, NUMBER::Imag,
                     detail::combine(mra, prec, {std::make_tuple(1.0, ri.get()), std::make_tuple(1.0, ir.get())}));
    else if (ri || ir)
        replace_part(out, NUMBER::Imag, ri ? std::move(ri) : std::move(ir));
}

// out = a * b with conjugation (mrcpp::cplxfunc::multiply(out, a, b, prec, absPrec, useMaxNorms)),
// e.g. rho_ij = phi_i^dagger phi_j (ExchangePotential.cpp:175).  out must not be conjugated.
inline void multiply(ComplexFunction &out, const ComplexFunction &a, const ComplexFunction &b, double prec,
                     bool absPrec = false, bool useMaxNorms = false) {
    if (out.conjugate()) throw Error(MW_ERR_ARG, "cplxfunc::multiply: conjugated output");
    multiply_real(out, a, b, prec, absPrec, useMaxNorms);
    multiply_imag(out, a, b, prec, absPrec, useMaxNorms);
}

// out = sum_i c_i inp_i on the union grid (mrcpp::cplxfunc::linear_combination, KAIN.cpp:170,182);
// Coefs: any vector of complex numbers with size() and operator[] (std::vector, Eigen::VectorXcd)
template <class Coefs>
void linear_combination(ComplexFunction &out, const Coefs &coefs, const std::vector<ComplexFunction> &inp,
                        double prec) {
    if ((size_t)coefs.size() != inp.size()) throw Error(MW_ERR_ARG, "linear_combination: size mismatch");
    if (out.conjugate()) throw Error(MW_ERR_ARG, "linear_combination: conjugated output");
    std::vector<std::tuple<double, FunctionTree<3> *>> re, im;
    for (size_t i = 0; i < inp.size(); i++) {
        const ComplexDouble c = coefs[i];
        const double t = inp[i].imagSign();
        FunctionTree<3> *x = inp[i].hasReal() ? &inp[i].real() : nullptr;
        FunctionTree<3> *y = inp[i].hasImag() ? &inp[i].imag() : nullptr;
        re.emplace_back(c.real(), x);
        re.emplace_back(-c.imag() * t, y);
        im.emplace_back(c.imag(), x);
        im.emplace_back(c.real() * t, y);
    }
    replace_part(out, NUMBER::Real, detail::combine(out.mra(), prec, re));
    replace_part(out, NUMBER::Imag, detail::combine(out.mra(), prec, im));
}

// mrcpp::cplxfunc::project(out, GaussExp, NUMBER::Real|Imag, prec)
inline void project(ComplexFunction &out, const GaussExp<3> &f, NUMBER type, double prec, bool absPrec = false) {
    if (type == NUMBER::Total) throw Error(MW_ERR_ARG, "cplxfunc::project: choose Real or Imag");
    out.alloc(type);
    FunctionTree<3> &t = type == NUMBER::Real ? out.real() : out.imag();
    t.clear();
    mrcpp::project(prec, t, f, -1, absPrec);
    if (type == NUMBER::Imag && out.conjugate()) t.rescale(-1.0);
}

// <a|b> = integral of conj(a) b (orbital::dot, src/qmfunctions/orbital_utils.cpp:79-82)
inline ComplexDouble dot(const ComplexFunction &a, const ComplexFunction &b) {
    // conj(a) = ar - i sa ai, b = br + i sb bi
    auto d = [](FunctionTree<3> &x, FunctionTree<3> &y) {
        double v = 0;
        check(mw_dot(x.handle(), y.handle(), &v), x.context());
        return v;
    };
    const double sa = a.imagSign(), sb = b.imagSign();
    double re = 0.0, im = 0.0;
    if (a.hasReal() && b.hasReal()) re += d(a.real(), b.real());
    if (a.hasImag() && b.hasImag()) re += sa * sb * d(a.imag(), b.imag());
    if (a.hasReal() && b.hasImag()) im += sb * d(a.real(), b.imag());
    if (a.hasImag() && b.hasReal()) im -= sa * d(a.imag(), b.real());
    return {re, im};
}

}  // namespace cplxfunc

}  // namespace mrcpp

// ---- GB300 batched entry above the mrcpp:: surface ----------------------------------------------
namespace mrcpp_gb300 {

// HelmholtzVector::operator() (src/scf_solver/HelmholtzVector.cpp:70-91 with apply(i, phi) at
// :141-159) as one batched call: out_i = H_i[phi_i] rescaled by -1/(2 pi), with mu_i =
// sqrt(-2 lambda_i) (lambda_i > 0 is an error, as MSG_ABORT "Mu cannot be complex" there),
// absolute precision, the real and imaginary parts of every orbital applied as separate jobs of one
// mw_apply_batch, the imaginary part's sign from the orbital's conjugation flag (+1/(2 pi) for a
// conjugated orbital, -1/(2 pi) otherwise).  `precision_mode` is MW_PREC_FP64 (the reference's) or a
// mixed mode; the operators are built together (mw_op_create_helmholtz_batch).
inline std::vector<mrcpp::ComplexFunction> helmholtz_vector(double prec, const std::vector<double> &lambda,
                                                            std::vector<mrcpp::ComplexFunction> &phi,
                                                            int precision_mode = MW_PREC_FP64) {
    using mrcpp::NUMBER;
    if (lambda.size() != phi.size()) throw mrcpp::Error(MW_ERR_ARG, "helmholtz_vector: size mismatch");
    std::vector<mrcpp::ComplexFunction> out;
    if (phi.empty()) return out;
    const auto &mra = phi[0].mra();
    const mw_ctx ctx = mra.handle();
    std::vector<double> mu(phi.size());
    for (size_t i = 0; i < phi.size(); i++) {
        if (lambda[i] > 0.0) throw mrcpp::Error(MW_ERR_ARG, "helmholtz_vector: mu cannot be complex (lambda > 0)");
        mu[i] = std::sqrt(-2.0 * lambda[i]);
    }
    std::vector<mw_op> ops(phi.size(), nullptr);
    mrcpp::check(mw_op_create_helmholtz_batch(ctx, (int)mu.size(), mu.data(), prec, ops.data()), ctx);
    struct OpGuard {
        std::vector<mw_op> &v;
        ~OpGuard() {
            for (mw_op o : v)
                if (o) mw_op_destroy(o);
        }
    } guard{ops};
    std::vector<mw_tree> outs, inps;
    std::vector<mw_op> jops;
    std::vector<double> scale;
    for (size_t i = 0; i < phi.size(); i++) {
        out.push_back(phi[i].paramCopy());
        const double pi = 3.14159265358979323846;
        if (phi[i].hasReal()) {
            out[i].alloc(NUMBER::Real);
            outs.push_back(out[i].real().handle());
            inps.push_back(phi[i].real().handle());
            jops.push_back(ops[i]);
            scale.push_back(-1.0 / (2.0 * pi));
        }
        if (phi[i].hasImag()) {
            out[i].alloc(NUMBER::Imag);
            outs.push_back(out[i].imag().handle());
            inps.push_back(phi[i].imag().handle());
            jops.push_back(ops[i]);
            scale.push_back((phi[i].conjugate() ? 1.0 : -1.0) / (2.0 * pi));
        }
    }
    if (outs.empty()) return out;
    std::vector<double> precs(outs.size(), prec);
    mrcpp::check(mw_apply_batch((int)outs.size(), precs.data(), outs.data(), jops.data(), inps.data(), nullptr, nullptr,
                                -1, 1, precision_mode),
                 ctx);
    for (size_t j = 0; j < outs.size(); j++) mrcpp::check(mw_tree_rescale(outs[j], scale[j]), ctx);
    return out;
}

}  // namespace mrcpp_gb300
