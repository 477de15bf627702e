// shim_check.cpp -- MRChem-shaped calls through include/mrcpp_gb300.hpp, compiled with g++ and
// linked against libmwgb300.so by tests/test_gpu_shim.py, which compares the trees this program
// writes with the CPU oracle.
//
//   argv[1]: output directory (trees written with mw_tree_save, one file per result)
//   stdout:  one JSON object of scalar results
//
// The call sequences follow the reference's call sites:
//   CoulombPotential::setupGlobalPotential   src/qmoperators/two_electron/CoulombPotential.cpp:115-160
//   HelmholtzVector::apply(i, phi)           src/scf_solver/HelmholtzVector.cpp:141-159
//   rho_ij = phi_i^dagger phi_j              src/qmoperators/two_electron/ExchangePotential.cpp:175
//   cplxfunc::linear_combination             src/scf_solver/KAIN.cpp:170,182
//   orbital::dot                             src/qmfunctions/orbital_utils.cpp:79-82
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "mrcpp_gb300.hpp"

using namespace mrcpp;

static std::string g_dir;

static void save(const FunctionTree<3> &t, const char *name) {
    check(mw_tree_save(t.handle(), (g_dir + "/" + name + ".mwt").c_str()), t.context());
}

static GaussExp<3> gauss(std::vector<GaussFunc<3>> fs) {
    GaussExp<3> e;
    for (auto &f : fs) e.append(f);
    return e;
}

// HelmholtzVector::apply(i, phi), src/scf_solver/HelmholtzVector.cpp:141-159, spelled as there
static ComplexFunction helmholtz_apply(const MultiResolutionAnalysis<3> &MRA, double lambda, double prec,
                                       ComplexFunction &phi) {
    double mu = std::sqrt(-2.0 * lambda);
    HelmholtzOperator H(MRA, mu, prec);
    ComplexFunction out = phi.paramCopy();
    const double pi = 3.14159265358979323846;
    if (phi.hasReal()) {
        out.alloc(NUMBER::Real);
        mrcpp::apply(prec, out.real(), H, phi.real(), -1, true);  // absolute prec
        out.real().rescale(-1.0 / (2.0 * pi));
    }
    if (phi.hasImag()) {
        out.alloc(NUMBER::Imag);
        mrcpp::apply(prec, out.imag(), H, phi.imag(), -1, true);
        double sign = (phi.conjugate()) ? 1.0 : -1.0;
        out.imag().rescale(sign / (2.0 * pi));
    }
    return out;
}

int main(int argc, char **argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: shim_check <outdir>\n");
        return 2;
    }
    g_dir = argv[1];
    const double prec = 1e-5;
    const double pi = 3.14159265358979323846;
    MultiResolutionAnalysis<3> MRA(BoundingBox<3>(-5, {-1, -1, -1}, {2, 2, 2}), InterpolatingBasis(7), 25);

    // ---- CoulombPotential::setupGlobalPotential: V = P[rho], rho = 4 normalized Gaussians ----
    const double al[4] = {0.7, 2.0, 6.5, 21.0};
    const std::array<double, 3> R[4] = {{0.3, -0.2, 0.1}, {-0.6, 0.5, 0.0}, {0.1, 0.9, -0.4}, {-0.2, -0.7, 0.6}};
    GaussExp<3> rho_exp;
    for (int i = 0; i < 4; i++) rho_exp.append(GaussFunc<3>(al[i], std::pow(al[i] / pi, 1.5), R[i]));
    FunctionTree<3> rho(MRA);
    mrcpp::project(prec, rho, rho_exp);
    PoissonOperator P(MRA, prec);
    FunctionTree<3> V(MRA);
    const double n_el = 4.0;
    mrcpp::apply(prec / n_el, V, P, rho);  // CoulombPotential.cpp:150-155: relative precision prec / N_el
    save(rho, "rho");
    save(V, "V");
    // the same apply with a second operator in mixed precision: the mode is per operator
    PoissonOperator Pm(MRA, prec);
    Pm.setPrecision(MW_PREC_MIXED);
    FunctionTree<3> Vm(MRA);
    mrcpp::apply(prec / n_el, Vm, Pm, rho);
    save(Vm, "Vm");
    double E = mrcpp::dot(rho, V);

    // an output that already holds coefficients is rejected (MSG_ERROR in CoulombPotential.cpp:122-123)
    bool rejected = false;
    try {
        mrcpp::apply(prec / n_el, V, P, rho);
    } catch (const mrcpp::Error &e) {
        rejected = e.code == MW_ERR_ARG || e.code == MW_ERR_STATE;
    }

    // ---- complex orbitals ----
    ComplexFunction phi(MRA), chi(MRA);
    cplxfunc::project(phi, gauss({GaussFunc<3>(1.2, 1.0, {0.2, 0.0, -0.1}), GaussFunc<3>(4.0, 0.3, {-0.3, 0.2, 0.1}, {1, 0, 0})}),
                      NUMBER::Real, prec);
    cplxfunc::project(phi, gauss({GaussFunc<3>(2.5, 0.6, {0.0, 0.3, 0.2}, {0, 1, 0})}), NUMBER::Imag, prec);
    cplxfunc::project(chi, gauss({GaussFunc<3>(0.8, 0.9, {-0.1, -0.2, 0.3})}), NUMBER::Real, prec);
    cplxfunc::project(chi, gauss({GaussFunc<3>(3.0, 0.5, {0.4, 0.1, -0.2}, {0, 0, 1})}), NUMBER::Imag, prec);
    save(phi.real(), "phi_re");
    save(phi.imag(), "phi_im");
    save(chi.real(), "chi_re");
    save(chi.imag(), "chi_im");

    // HelmholtzVector::apply(i, phi) on phi and on phi^dagger (the imaginary part's sign flips)
    ComplexFunction phid = phi.dagger();
    ComplexFunction h0 = helmholtz_apply(MRA, -0.5, prec, phi);
    ComplexFunction h1 = helmholtz_apply(MRA, -0.5, prec, phid);
    save(h0.real(), "h0_re");
    save(h0.imag(), "h0_im");
    save(h1.real(), "h1_re");
    save(h1.imag(), "h1_im");
    // the batched replacement of HelmholtzVector::operator(): the same orbitals in one call
    std::vector<ComplexFunction> vin = {phi, phid, chi};
    std::vector<ComplexFunction> hv = mrcpp_gb300::helmholtz_vector(prec, {-0.5, -0.5, -1.2}, vin);
    save(hv[0].real(), "hv0_re");
    save(hv[0].imag(), "hv0_im");
    save(hv[1].imag(), "hv1_im");
    save(hv[2].real(), "hv2_re");
    save(hv[2].imag(), "hv2_im");

    // rho_ij = phi^dagger chi (ExchangePotential.cpp:175: prec_m1, absPrec, useMaxNorms)
    ComplexFunction rho_ij = phi.paramCopy();
    cplxfunc::multiply(rho_ij, phi.dagger(), chi, prec / 10, true, true);
    save(rho_ij.real(), "rhoij_re");
    save(rho_ij.imag(), "rhoij_im");

    // KAIN-style linear combination of phi^dagger and chi with complex coefficients
    std::vector<ComplexDouble> coefs = {{0.5, -1.0}, {2.0, 0.25}};
    ComplexFunction lc = phi.paramCopy();
    cplxfunc::linear_combination(lc, coefs, std::vector<ComplexFunction>{phi.dagger(), chi}, prec);
    save(lc.real(), "lc_re");
    save(lc.imag(), "lc_im");

    // <phi|chi>, and <phi| i phi> = i |phi|^2 through ComplexFunction::add and a complex rescale
    ComplexDouble d = cplxfunc::dot(phi, chi);
    ComplexFunction iphi = phi.paramCopy();
    iphi.add({1.0, 0.0}, phi);
    iphi.rescale(ComplexDouble(0.0, 1.0));
    ComplexDouble d2 = cplxfunc::dot(phi, iphi);
    // the same through a conjugated accumulator: (phi^dagger)^dagger = phi
    ComplexFunction acc = phi.paramCopy().dagger();
    acc.add({1.0, 0.0}, phi);
    ComplexDouble d3 = cplxfunc::dot(phi, acc.dagger().dagger());

    std::printf("{\"E_coulomb\": %.17g, \"rejected_nonempty_output\": %s, \"dot_phi_chi\": [%.17g, %.17g], "
                "\"dot_phi_iphi\": [%.17g, %.17g], \"dot_phi_acc\": [%.17g, %.17g], \"phi_sqnorm\": %.17g, "
                "\"nnodes\": {\"rho\": %d, \"V\": %d, \"phi\": %d}}\n",
                E, rejected ? "true" : "false", d.real(), d.imag(), d2.real(), d2.imag(), d3.real(), d3.imag(),
                phi.squaredNorm(), rho.getNNodes(), V.getNNodes(), phi.getNNodes(NUMBER::Total));
    return 0;
}
