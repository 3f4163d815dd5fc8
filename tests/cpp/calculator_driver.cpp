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

}  // extern "C"
