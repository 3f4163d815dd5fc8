// Test driver of the C++ host layer (include/dsf_calculator.hpp): the
// reference-shaped calls on one HC structure, driven from
// tests/test_cpp_host.py through one extern "C" entry.
#include "dsf_calculator.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

namespace {
std::string g_err;
}

extern "C" {

const char *drv_error() { return g_err.c_str(); }

// atoms: xyz [n][3], adp [n][6] (first nadp used), occ [n]; hkl [m][3], dtdf [m][2]; include [n] (0/1)
// outputs: f [m][2] and the derivatives [n][3], [n][6], [n] of the whole-set call; f_only [m][2] of
// calculateStructureFactors; f1 [2], d1_xyz [n][3][2], d1_adp [n][6][2], d1_occ [n][2] of the single-h call at
// hkl[0]; ff [n][2] of calculateFormFactors at hkl[1]; checks setAnomalous, the DerivativesSelector overload and getModelInformation itself
int drv_hc(int device, const dsf_symmetry *sym, const dsf_hc_model *model, const dsf_atoms *atoms, int precision,
           const double *xyz, const double *adp, const double *occ, int m, const int *hkl, const double *dtdf,
           const int *include, double *f, double *d_xyz, double *d_adp, double *d_occ, double *f_only, double *f1,
           double *d1_xyz, double *d1_adp, double *d1_occ, double *ff)
{
    try {
        auto engine = std::make_shared<dsf::Engine>(device);
        dsf::HcCalculator calc(engine, *sym, *model, *atoms);
        calc.setPrecision(precision);
        calc.setN_threads(8);
        const int n = atoms->n_atoms;
        std::vector<dsf::AtomInCrystal> at(n);
        for (int a = 0; a < n; a++) {
            at[a].coordinates = {xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]};
            at[a].adp.assign(adp + 6 * a, adp + 6 * a + atoms->adp_components[a]);
            at[a].occupancy = occ[a];
        }
        std::vector<dsf::Vector3i> h(m);
        std::vector<dsf::cplx> g(m);
        for (int i = 0; i < m; i++) {
            h[i] = {hkl[3 * i], hkl[3 * i + 1], hkl[3 * i + 2]};
            g[i] = dsf::cplx(dtdf[2 * i], dtdf[2 * i + 1]);
        }
        std::vector<bool> count(n);
        for (int a = 0; a < n; a++) count[a] = include[a] != 0;
        std::vector<dsf::cplx> fv;
        std::vector<dsf::TargetFunctionAtomicParamDerivatives> d;
        calc.calculateStructureFactorsAndDerivatives(at, h, fv, d, g, count);
        std::memcpy(f, fv.data(), sizeof(double) * 2 * m);
        for (int a = 0; a < n; a++) {
            for (int k = 0; k < 3; k++) d_xyz[3 * a + k] = d[a].atomic_position_derivatives[k];
            for (int k = 0; k < 6; k++) d_adp[6 * a + k] = k < (int)d[a].adp_derivatives.size() ? d[a].adp_derivatives[k] : 0.0;
            d_occ[a] = d[a].occupancy_derivatives;
        }
        std::vector<dsf::cplx> f2;
        calc.calculateStructureFactors(at, h, f2, count);
        std::memcpy(f_only, f2.data(), sizeof(double) * 2 * m);
        dsf::cplx fs;
        dsf::SfDerivativesAtHkl ds;
        calc.calculateStructureFactorsAndDerivatives(h[0], fs, ds, count);
        f1[0] = fs.real();
        f1[1] = fs.imag();
        for (int a = 0; a < n; a++) {
            for (int k = 0; k < 3; k++) {
                d1_xyz[6 * a + 2 * k] = ds.atomicPostionDerivatives[a][k].real();
                d1_xyz[6 * a + 2 * k + 1] = ds.atomicPostionDerivatives[a][k].imag();
            }
            for (int k = 0; k < 6; k++) {
                const bool have = k < (int)ds.adpDerivatives[a].size();
                d1_adp[12 * a + 2 * k] = have ? ds.adpDerivatives[a][k].real() : 0.0;
                d1_adp[12 * a + 2 * k + 1] = have ? ds.adpDerivatives[a][k].imag() : 0.0;
            }
            d1_occ[2 * a] = ds.occupancyDerivatives[a].real();
            d1_occ[2 * a + 1] = ds.occupancyDerivatives[a].imag();
        }
        std::vector<dsf::cplx> ffv;
        calc.calculateFormFactors(h[1], ffv, count);
        std::memcpy(ff, ffv.data(), sizeof(double) * 2 * n);
        // the whole set again after the single-h call: the resident set was restored
        std::vector<dsf::cplx> f3;
        calc.calculateStructureFactors(at, h, f3, count);
        for (int i = 0; i < m; i++)
            if (std::abs(f3[i] - f2[i]) > 1e-9 * (1.0 + std::abs(f2[i]))) throw dsf::Error("set not restored");
        // setAnomalous: zero f', f'' changes F, the creation values bring it back
        if (atoms->anomalous) {
            calc.setAnomalous(std::vector<dsf::cplx>(n, dsf::cplx(0.0, 0.0)));
            calc.calculateStructureFactors(at, h, f3, count);
            double diff = 0.0;
            for (int i = 0; i < m; i++) diff = std::max(diff, std::abs(f3[i] - f2[i]));
            if (diff == 0.0) throw dsf::Error("setAnomalous had no effect");
            std::vector<dsf::cplx> an(n);
            for (int a = 0; a < n; a++) an[a] = dsf::cplx(atoms->anomalous[2 * a], atoms->anomalous[2 * a + 1]);
            calc.setAnomalous(an);
            calc.calculateStructureFactors(at, h, f3, count);
            for (int i = 0; i < m; i++)
                if (std::abs(f3[i] - f2[i]) > 1e-9 * (1.0 + std::abs(f2[i]))) throw dsf::Error("setAnomalous not restored");
        }
        // DerivativesSelector: positions only; F and dF/dxyz as the full call, the other classes zero
        {
            dsf::DerivativesSelector sel;
            sel.d_adp = sel.d_occ = false;
            std::vector<dsf::cplx> fsel;
            std::vector<dsf::TargetFunctionAtomicParamDerivatives> dsel;
            calc.calculateStructureFactorsAndDerivatives(at, h, fsel, dsel, g, count, sel);
            for (int i = 0; i < m; i++)
                if (std::abs(fsel[i] - fv[i]) > 1e-9 * (1.0 + std::abs(fv[i]))) throw dsf::Error("selector: F differs");
            for (int a = 0; a < n; a++) {
                for (int k = 0; k < 3; k++)
                    if (std::abs(dsel[a].atomic_position_derivatives[k] - d[a].atomic_position_derivatives[k]) >
                        1e-9 * (1.0 + std::abs(d[a].atomic_position_derivatives[k])))
                        throw dsf::Error("selector: dF/dxyz differs");
                for (double v : dsel[a].adp_derivatives)
                    if (v != 0.0) throw dsf::Error("selector: unselected ADP derivative not zero");
                if (dsel[a].occupancy_derivatives != 0.0) throw dsf::Error("selector: unselected occupancy derivative");
            }
        }
        std::vector<std::pair<std::string, std::string> > info;
        calc.getModelInformation(info);
        if (info.size() != 1 || info[0].second != "Hansen-Coppens multipole model") throw dsf::Error("model information");
        // an error of the reference's kind: mismatched dT/dF size
        try {
            std::vector<dsf::cplx> bad(m + 1);
            calc.calculateStructureFactorsAndDerivatives(at, h, fv, d, bad, count);
            throw dsf::Error("size mismatch not rejected");
        } catch (const dsf::Error &ex) {
            if (std::string(ex.what()).find("sizes differ") == std::string::npos) throw;
        }
        return 0;
    } catch (const std::exception &ex) {
        g_err = ex.what();
        return 1;
    }
}

// XD-style definitions from the flat arrays of the golden fixtures (lcs_def [n][7] = central, axis1, axis2,
// right-handed, n1, n2a, n2b; lcs_atoms consumed in order; lcs_dummy [n][3][3] fractional)
static std::vector<dsf::XdLcs> lcs_definitions(int n, const int *def, const int *list, const double *dummy)
{
    std::vector<dsf::XdLcs> out(n);
    int cursor = 0;
    for (int a = 0; a < n; a++) {
        const int *d = def + 7 * a;
        dsf::XdLcs &q = out[a];
        q.central = d[0];
        q.axis1 = d[1];
        q.axis2 = d[2];
        q.right_handed = d[3] != 0;
        std::vector<int> *pts[3] = {&q.point1, &q.point2_from, &q.point2_to};
        dsf::Vector3d *dum[3] = {&q.dummy1, &q.dummy2_from, &q.dummy2_to};
        for (int p = 0; p < 3; p++) {
            for (int k = 0; k < d[4 + p]; k++) pts[p]->push_back(list[cursor++]);
            for (int k = 0; k < 3; k++) (*dum[p])[k] = dummy[9 * a + 3 * p + k];
        }
    }
    return out;
}

static std::vector<dsf::AtomInCrystal> atom_list(int n, const int *nadp, const double *xyz, const double *adp,
                                                 const double *occ)
{
    std::vector<dsf::AtomInCrystal> at(n);
    for (int a = 0; a < n; a++) {
        at[a].coordinates = {xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]};
        at[a].adp.assign(adp + 6 * a, adp + 6 * a + nadp[a]);
        at[a].occupancy = occ[a];
    }
    return at;
}

// host only: the LCS matrices ([n][9]) of the definitions for the positions xyz (crystal convention)
int drv_lcs_matrices(int n, const double *cell, int cartesian, const double *xyz, const int *def, const int *list,
                     const double *dummy, double *out)
{
    try {
        const auto defs = lcs_definitions(n, def, list, dummy);
        std::vector<dsf::AtomInCrystal> at(n);
        for (int a = 0; a < n; a++) at[a].coordinates = {xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]};
        const auto M = dsf::fractionalToCartesian(cell);
        for (int a = 0; a < n; a++) {
            const auto m = dsf::lcsMatrix(defs[a], M, cartesian != 0, at);
            std::copy(m.begin(), m.end(), out + 9 * a);
        }
        return 0;
    } catch (const std::exception &ex) {
        g_err = ex.what();
        return 1;
    }
}

// AnyHcCalculator's flow with local coordinate systems: the calculator is created on the atoms of `atoms`
// (xyz), the definitions are set (frozen or not), and the whole-set call is made with the atoms at xyz_moved;
// outputs F and derivatives of that call and the matrices the engine holds afterwards (lcs_out [n][9])
int drv_hc_lcs(int device, const dsf_symmetry *sym, const dsf_hc_model *model, const dsf_atoms *atoms,
               int precision, int frozen, const double *xyz, const double *xyz_moved, const double *adp,
               const double *occ, const int *def, const int *list, const double *dummy, int m, const int *hkl,
               const double *dtdf, double *f, double *d_xyz, double *d_adp, double *d_occ, double *lcs_out)
{
    try {
        auto engine = std::make_shared<dsf::Engine>(device);
        dsf::HcCalculator calc(engine, *sym, *model, *atoms);
        calc.setPrecision(precision);
        const int n = atoms->n_atoms;
        calc.setLocalCoordinateSystems(lcs_definitions(n, def, list, dummy), frozen != 0,
                                       atom_list(n, atoms->adp_components, xyz, adp, occ));
        const auto moved = atom_list(n, atoms->adp_components, xyz_moved, adp, occ);
        std::vector<dsf::Vector3i> h(m);
        std::vector<dsf::cplx> g(m);
        for (int i = 0; i < m; i++) {
            h[i] = {hkl[3 * i], hkl[3 * i + 1], hkl[3 * i + 2]};
            g[i] = dsf::cplx(dtdf[2 * i], dtdf[2 * i + 1]);
        }
        std::vector<dsf::cplx> fv;
        std::vector<dsf::TargetFunctionAtomicParamDerivatives> d;
        calc.calculateStructureFactorsAndDerivatives(moved, h, fv, d, g);
        std::memcpy(f, fv.data(), sizeof(double) * 2 * m);
        for (int a = 0; a < n; a++) {
            for (int k = 0; k < 3; k++) d_xyz[3 * a + k] = d[a].atomic_position_derivatives[k];
            for (int k = 0; k < 6; k++) d_adp[6 * a + k] = k < (int)d[a].adp_derivatives.size() ? d[a].adp_derivatives[k] : 0.0;
            d_occ[a] = d[a].occupancy_derivatives;
        }
        std::copy(calc.localCoordinateSystems().begin(), calc.localCoordinateSystems().end(), lcs_out);
        return 0;
    } catch (const std::exception &ex) {
        g_err = ex.what();
        return 1;
    }
}

// CombinedCalculator over an HC part (hc_* descriptors of the structure of the atoms hc_idx) and an IAM part
// (iam_* descriptors of the atoms iam_idx); the whole structure's atoms: xyz [n][3], adp [n][6], occ [n], nadp [n]
int drv_combined(int device, int precision, const dsf_symmetry *hc_sym, const dsf_hc_model *hc_model,
                 const dsf_atoms *hc_atoms, const int *hc_idx, const dsf_symmetry *iam_sym,
                 const dsf_iam_model *iam_model, const dsf_atoms *iam_atoms, const int *iam_idx, int n,
                 const int *nadp, const double *xyz, const double *adp, const double *occ, int m, const int *hkl,
                 const double *dtdf, double *f, double *d_xyz, double *d_adp, double *d_occ)
{
    try {
        auto engine = std::make_shared<dsf::Engine>(device);
        auto hc = std::make_shared<dsf::HcCalculator>(engine, *hc_sym, *hc_model, *hc_atoms);
        auto iam = std::make_shared<dsf::IamCalculator>(engine, *iam_sym, *iam_model, *iam_atoms, "IT92");
        dsf::CombinedCalculator comb({hc, iam}, {std::vector<int>(hc_idx, hc_idx + hc_atoms->n_atoms),
                                                 std::vector<int>(iam_idx, iam_idx + iam_atoms->n_atoms)});
        comb.setPrecision(precision);
        const auto at = atom_list(n, nadp, xyz, adp, occ);
        std::vector<dsf::Vector3i> h(m);
        std::vector<dsf::cplx> g(m);
        for (int i = 0; i < m; i++) {
            h[i] = {hkl[3 * i], hkl[3 * i + 1], hkl[3 * i + 2]};
            g[i] = dsf::cplx(dtdf[2 * i], dtdf[2 * i + 1]);
        }
        std::vector<dsf::cplx> fv;
        std::vector<dsf::TargetFunctionAtomicParamDerivatives> d;
        comb.calculateStructureFactorsAndDerivatives(at, h, fv, d, g, std::vector<bool>(n, true));
        std::memcpy(f, fv.data(), sizeof(double) * 2 * m);
        for (int a = 0; a < n; a++) {
            for (int k = 0; k < 3; k++) d_xyz[3 * a + k] = d[a].atomic_position_derivatives[k];
            for (int k = 0; k < 6; k++) d_adp[6 * a + k] = k < (int)d[a].adp_derivatives.size() ? d[a].adp_derivatives[k] : 0.0;
            d_occ[a] = d[a].occupancy_derivatives;
        }
        return 0;
    } catch (const std::exception &ex) {
        g_err = ex.what();
        return 1;
    }
}

}  // extern "C"
