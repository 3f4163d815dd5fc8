// Drives the reference library's own CPU structure-factor code for parity
// pinning.  TEST INFRASTRUCTURE: compiled only by oracle/Makefile.ref
// together with the reference sources where they lie; used by
// tests/golden/make_golden.py to write golden fixtures and by the CPU
// tests to pin the oracle restatement.  Nothing in the shipped library
// links it.
//
// Entry points build the reference's own objects and call:
//   * HansenCoppensStructureFactorCalculator + setCalculationMode("CPU")
//     (src/Scattering/HansenCoppensStructureFactorCalculator.cpp:380-508,
//      engine HansenCoppens_SF_Engine3) -- the HC path;
//   * AnyScattererStructureFactorCalculator + IamFormFactorCalculationsManager
//     (the AnyIamCalculator path, src/Scattering/AnyIamCalculator.cpp:49-154);
//   * AnyScattererStructureFactorCalculator + ConstFormFactorCalculationsManager
//     (the tabulated path behind TscFileBasedSfCalculator).
#include "discamb/BasicChemistry/periodic_table.h"
#include "discamb/CrystalStructure/Crystal.h"
#include "discamb/CrystalStructure/SpaceGroup.h"
#include "discamb/CrystalStructure/SpaceGroupOperation.h"
#include "discamb/CrystalStructure/UnitCell.h"
#include "discamb/HC_Model/HC_ModelParameters.h"
#include "discamb/HC_Model/XdLocalCoordinateSystem.h"
#include "discamb/Scattering/AnyHcCalculator.h"
#include "discamb/Scattering/AnyIamCalculator.h"
#include "discamb/Scattering/CombinedStructureFactorCalculator.h"
#include "discamb/IO/tsc_io.h"
#include "discamb/Scattering/AnyScattererStructureFactorCalculator.h"
#include "discamb/Scattering/ConstFormFactorCalculationsManager.h"
#include "discamb/Scattering/HansenCoppensStructureFactorCalculator.h"
#include "discamb/Scattering/IamFormFactorCalculationsManager.h"
#include "discamb/Scattering/NGaussianFormFactorsTable.h"

#include <chrono>
#include <complex>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

using namespace discamb;
using std::complex;
using std::string;
using std::vector;

namespace {

std::string g_last_error;

struct Input {
    const double *cell;
    const char *ops;          // ';' separated operation strings
    int n_atoms;
    const double *xyz;        // fractional
    const int *n_adp;
    const double *adp;        // U_cif / Uiso, 6 per atom
    const double *occ;
    const int *mult;
    const char *atom_types;   // ';' separated element labels (IAM / labels)
};

// conventions of the crystal the following calls build (the inputs are given in them and the reference returns
// the derivatives in them, HansenCoppensStructureFactorCalculator.cpp:69-70, 634-664;
// AnyScattererStructureFactorCalculator.cpp:89-90): xyz fractional (0) or Cartesian (1); ADPs U_cif (0), U_cart (1)
// or U_star (2)
int g_xyz_cartesian = 0;
int g_adp_convention = 0;

Crystal make_crystal(const Input &in)
{
    Crystal c;
    c.unitCell.set(in.cell[0], in.cell[1], in.cell[2], in.cell[3], in.cell[4], in.cell[5]);
    vector<SpaceGroupOperation> ops;
    std::stringstream ss(in.ops);
    string item;
    while (std::getline(ss, item, ';'))
        if (!item.empty()) ops.push_back(SpaceGroupOperation(item));
    c.spaceGroup.set(ops);
    vector<string> labels;
    if (in.atom_types) {
        std::stringstream ls(in.atom_types);
        while (std::getline(ls, item, ';')) labels.push_back(item);
    }
    c.atoms.resize(in.n_atoms);
    for (int i = 0; i < in.n_atoms; i++) {
        AtomInCrystal &a = c.atoms[i];
        a.coordinates = Vector3d(in.xyz[3 * i], in.xyz[3 * i + 1], in.xyz[3 * i + 2]);
        a.adp.assign(in.adp + 6 * i, in.adp + 6 * i + in.n_adp[i]);
        a.occupancy = in.occ[i];
        a.multiplicity = in.mult[i];
        if (i < (int)labels.size()) { a.type = labels[i]; a.label = labels[i] + std::to_string(i + 1); }
    }
    c.adpConvention = g_adp_convention == 1 ? structural_parameters_convention::AdpConvention::U_cart
                      : g_adp_convention == 2 ? structural_parameters_convention::AdpConvention::U_star
                                              : structural_parameters_convention::AdpConvention::U_cif;
    c.xyzCoordinateSystem = g_xyz_cartesian ? structural_parameters_convention::XyzCoordinateSystem::cartesian
                                            : structural_parameters_convention::XyzCoordinateSystem::fractional;
    return c;
}

void write_out(const vector<complex<double> > &f, const vector<TargetFunctionAtomicParamDerivatives> &d,
               double *f_out, double *d_xyz, double *d_adp, double *d_occ)
{
    for (size_t i = 0; i < f.size(); i++) { f_out[2 * i] = f[i].real(); f_out[2 * i + 1] = f[i].imag(); }
    for (size_t a = 0; a < d.size(); a++) {
        for (int j = 0; j < 3; j++) d_xyz[3 * a + j] = d[a].atomic_position_derivatives[j];
        for (int j = 0; j < 6; j++) d_adp[6 * a + j] = j < (int)d[a].adp_derivatives.size() ? d[a].adp_derivatives[j] : 0.0;
        d_occ[a] = d[a].occupancy_derivatives;
    }
}

// the reference's HC model parameters from flat arrays (wavefunctions as Slater orbitals: per wfn
// [orb_off[w], orb_off[w+1]) orbitals, per orbital [sto_off[o], sto_off[o+1]) Slater functions)
HC_ModelParameters make_hc_params(int n_atoms, const int *atom_wfn, const int *atom_type, int n_wfn, const int *orb_off,
                                  const int *orb_occ, const int *orb_core, const int *sto_off, const int *sto_pow,
                                  const double *sto_exp, const double *sto_coeff, const double *def_exp,
                                  const int *def_npow, const int *def_pow, const double *wfn_anom, const int *wfn_z,
                                  int n_types, const int *type_nl, const double *type_plm, const double *type_pval,
                                  const double *type_kappa, const double *type_kappa_p)
{
    HC_ModelParameters p;
    p.wfn_parameters.resize(n_wfn);
    for (int w = 0; w < n_wfn; w++) {
        HC_WfnType &wt = p.wfn_parameters[w];
        wt.wfnAtomTypeName = "W" + std::to_string(w);
        wt.atomic_number = wfn_z[w];
        for (int o = orb_off[w]; o < orb_off[w + 1]; o++) {
            SlaterTypeAtomicOrbitalRdf orb;
            for (int s = sto_off[o]; s < sto_off[o + 1]; s++) {
                orb.power_r.push_back(sto_pow[s]);
                orb.exponents.push_back(sto_exp[s]);
                orb.coefficients.push_back(sto_coeff[s]);
            }
            int idx = (int)wt.orbitals.size();
            wt.orbitals.push_back(orb);
            wt.orbital_occupancy.push_back(orb_occ[o]);
            if (orb_core[o]) wt.core_orbitals_indices.push_back(idx);
            else wt.valence_orbitals_indices.push_back(idx);
        }
        wt.deformation_valence_exponent = def_exp[w];
        wt.deformation_valence_power.assign(def_pow + 5 * w, def_pow + 5 * w + def_npow[w]);
        wt.anomalous_scattering = complex<double>(wfn_anom[2 * w], wfn_anom[2 * w + 1]);
    }
    p.type_parameters.resize(n_types);
    for (int t = 0; t < n_types; t++) {
        HC_AtomTypeParameters &tp = p.type_parameters[t];
        tp.p_lm.resize(type_nl[t]);
        for (int l = 0; l < type_nl[t]; l++)
            tp.p_lm[l].assign(type_plm + 25 * t + l * l, type_plm + 25 * t + l * l + 2 * l + 1);
        tp.p_val = type_pval[t];
        tp.kappa_spherical_valence = type_kappa[t];
        tp.kappa_deformation_valence = type_kappa_p[t];
    }
    p.atom_to_wfn_map.assign(atom_wfn, atom_wfn + n_atoms);
    p.atom_to_type_map.assign(atom_type, atom_type + n_atoms);
    return p;
}

// XD-style local coordinate systems from flat arrays (lcs_def [n][7] = central, axis 1, axis 2 (+-1..3 for
// +-X..Z), right-handed, n1, n2a, n2b; the points are sums of the atoms listed in lcs_atoms (consumed in order)
// or, with n = 0, the fractional dummy position lcs_dummy[a][point][3])
vector<std::shared_ptr<LocalCoordinateSystemInCrystal> > make_xd_lcs(const Crystal &crystal,
                                                                      const vector<string> &labels, int n_atoms,
                                                                      const int *lcs_def, const int *lcs_atoms,
                                                                      const double *lcs_dummy)
{
    const char *axes[] = {"-Z", "-Y", "-X", "", "X", "Y", "Z"};
    vector<std::shared_ptr<LocalCoordinateSystemInCrystal> > lcs;
    int cursor = 0;
    for (int a = 0; a < n_atoms; a++) {
        const int *d = lcs_def + 7 * a;
        vector<Vector3d> dummies;
        string pts[3];
        for (int q = 0; q < 3; q++) {
            const int cnt = d[4 + q];
            if (cnt == 0) {
                pts[q] = "DUM" + std::to_string(dummies.size());
                const double *v = lcs_dummy + 9 * a + 3 * q;
                dummies.push_back(Vector3d(v[0], v[1], v[2]));
            } else {
                for (int k = 0; k < cnt; k++) pts[q] += (k ? ";" : "") + labels[lcs_atoms[cursor++]];
            }
        }
        auto x = std::make_shared<XdLocalCoordinateSystem>();
        x->set(labels[d[0]], pts[0], pts[1], pts[2], axes[d[1] + 3], axes[d[2] + 3], d[3] != 0, crystal, true,
               dummies);
        lcs.push_back(x);
    }
    return lcs;
}

} // namespace

extern "C" {

const char *ref_last_error(void) { return g_last_error.c_str(); }

int ref_set_conventions(int xyz_cartesian, int adp_convention)
{
    g_xyz_cartesian = xyz_cartesian != 0;
    g_adp_convention = adp_convention;
    return 0;
}

// electron scattering (Mott-Bethe conversion inside the engine) for the following ref_hc_sf calls
static bool g_electron = false;
int ref_set_electron(int on)
{
    g_electron = on != 0;
    return 0;
}

// point-group-symmetrised deformation valence (HansenCoppens_SF_EngineSymm instead of Engine3, selected by
// set_def_val_symm, HansenCoppensStructureFactorCalculator.cpp:447-468) for the following ref_hc_sf calls
static bool g_def_val_symm = false;
int ref_set_def_val_symm(int on)
{
    g_def_val_symm = on != 0;
    return 0;
}

// single-h form factors: while set, ref_hc_sf and ref_iam_sf also write calculateFormFactors(h_i) for every
// input reflection into g_ff_out ([n_hkl][n_atoms][re, im], include mask of the call)
static double *g_ff_out = nullptr;
int ref_set_form_factor_out(double *ff_out)
{
    g_ff_out = ff_out;
    return 0;
}

// Hansen-Coppens path through HansenCoppensStructureFactorCalculator ("CPU").
// Wavefunctions as Slater orbitals: per wfn [orb_off[w], orb_off[w+1]) orbitals,
// per orbital [sto_off[o], sto_off[o+1]) Slater functions.
int ref_hc_sf(const double *cell, const char *ops, int n_atoms, const double *xyz, const int *n_adp,
              const double *adp, const double *occ, const int *mult, const int *atom_wfn,
              const int *atom_type, const double *lcs,
              int n_wfn, const int *orb_off, const int *orb_occ, const int *orb_core,
              const int *sto_off, const int *sto_pow, const double *sto_exp, const double *sto_coeff,
              const double *def_exp, const int *def_npow, const int *def_pow, const double *wfn_anom,
              const int *wfn_z,
              int n_types, const int *type_nl, const double *type_plm, const double *type_pval,
              const double *type_kappa, const double *type_kappa_p,
              int n_hkl, const int *hkl, const double *dtdf, const double *atom_anom, const int *include,
              int n_threads, double *f_out, double *d_xyz, double *d_adp, double *d_occ, double *ms)
{
    try {
        // atom type labels = element symbols of the atoms' wavefunctions (the engine takes the atomic numbers
        // for electron scattering from them, crystal_structure_utilities::atomicNumbers)
        std::string types;
        for (int a = 0; a < n_atoms; a++) types += periodic_table::symbol(wfn_z[atom_wfn[a]]) + ";";
        Input in{cell, ops, n_atoms, xyz, n_adp, adp, occ, mult, types.c_str()};
        Crystal crystal = make_crystal(in);
        HC_ModelParameters p = make_hc_params(n_atoms, atom_wfn, atom_type, n_wfn, orb_off, orb_occ, orb_core, sto_off,
                                              sto_pow, sto_exp, sto_coeff, def_exp, def_npow, def_pow, wfn_anom, wfn_z,
                                              n_types, type_nl, type_plm, type_pval, type_kappa, type_kappa_p);
        vector<Matrix3d> lcsm(n_atoms);
        for (int a = 0; a < n_atoms; a++)
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) lcsm[a](i, j) = lcs[9 * a + 3 * i + j];
        HansenCoppensStructureFactorCalculator calc(crystal, p);
        calc.setCalculationMode("CPU");
        calc.setN_Threads(n_threads);
        calc.setElectronScattering(g_electron);
        calc.set_def_val_symm(g_def_val_symm);
        if (atom_anom) {
            vector<complex<double> > an(n_atoms);
            for (int a = 0; a < n_atoms; a++) an[a] = complex<double>(atom_anom[2 * a], atom_anom[2 * a + 1]);
            calc.set_anomalous_dispersion_per_atom(an);
        }
        vector<Vector3i> h(n_hkl);
        vector<complex<double> > g(n_hkl), f;
        for (int i = 0; i < n_hkl; i++) {
            h[i] = Vector3i(hkl[3 * i], hkl[3 * i + 1], hkl[3 * i + 2]);
            g[i] = complex<double>(dtdf[2 * i], dtdf[2 * i + 1]);
        }
        vector<bool> inc(n_atoms, true);
        if (include) for (int a = 0; a < n_atoms; a++) inc[a] = include[a] != 0;
        vector<TargetFunctionAtomicParamDerivatives> d;
        auto t0 = std::chrono::steady_clock::now();
        calc.calculateStructureFactorsAndDerivatives(crystal.atoms, lcsm, h, f, d, g, inc);
        auto t1 = std::chrono::steady_clock::now();
        if (g_ff_out) {
            vector<complex<double> > ff;
            for (int i = 0; i < n_hkl; i++) {
                calc.calculateFormFactors(lcsm, h[i], ff, inc);
                for (int a = 0; a < n_atoms; a++) {
                    g_ff_out[2 * ((size_t)i * n_atoms + a)] = ff[a].real();
                    g_ff_out[2 * ((size_t)i * n_atoms + a) + 1] = ff[a].imag();
                }
            }
        }
        if (ms) *ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        write_out(f, d, f_out, d_xyz, d_adp, d_occ);
        return 0;
    } catch (const std::exception &ex) {
        g_last_error = ex.what();
        return 1;
    } catch (...) {
        g_last_error = "unknown exception";
        return 1;
    }
}

// Gaussian coefficients the reference's IAM table holds for a label.
int ref_iam_coefficients(const char *label, const char *table, double *a, double *b, double *c, int *n)
{
    try {
        if (!n_gaussian_form_factors_table::hasFormFactor(label, table)) return 1;
        NGaussianFormFactor ff = n_gaussian_form_factors_table::getFormFactor(label, table);
        vector<double> va, vb;
        ff.get_parameters(va, vb, *c);
        *n = (int)va.size();
        for (int i = 0; i < *n && i < 5; i++) { a[i] = va[i]; b[i] = vb[i]; }
        return 0;
    } catch (const std::exception &ex) {
        g_last_error = ex.what();
        return 1;
    } catch (...) {
        g_last_error = "unknown exception";
        return 1;
    }
}

// IAM path of AnyIamCalculator: AnyScatterer engine over all operations with
// n-Gaussian form factors from the named table.
int ref_iam_sf(const double *cell, const char *ops, const char *labels, const char *table, int n_atoms,
               const double *xyz, const int *n_adp, const double *adp, const double *occ, const int *mult,
               int n_hkl, const int *hkl, const double *dtdf, int n_threads,
               double *f_out, double *d_xyz, double *d_adp, double *d_occ, double *ms)
{
    try {
        Input in{cell, ops, n_atoms, xyz, n_adp, adp, occ, mult, labels};
        Crystal crystal = make_crystal(in);
        AnyScattererStructureFactorCalculator calc(crystal);
        std::shared_ptr<AtomicFormFactorCalculationsManager> mgr =
            std::make_shared<IamFormFactorCalculationsManager>(crystal, string(table));
        calc.setAtomicFormfactorManager(mgr);
        vector<Vector3i> h(n_hkl);
        vector<complex<double> > g(n_hkl), f;
        for (int i = 0; i < n_hkl; i++) {
            h[i] = Vector3i(hkl[3 * i], hkl[3 * i + 1], hkl[3 * i + 2]);
            g[i] = complex<double>(dtdf[2 * i], dtdf[2 * i + 1]);
        }
        vector<bool> inc(n_atoms, true);
        vector<TargetFunctionAtomicParamDerivatives> d;
        auto t0 = std::chrono::steady_clock::now();
        calc.calculateStructureFactorsAndDerivatives(h, f, d, g, inc);
        auto t1 = std::chrono::steady_clock::now();
        if (g_ff_out) {
            vector<complex<double> > ff;
            for (int i = 0; i < n_hkl; i++) {
                calc.calculateFormFactors(h[i], ff, inc);
                for (int a = 0; a < n_atoms; a++) {
                    g_ff_out[2 * ((size_t)i * n_atoms + a)] = ff[a].real();
                    g_ff_out[2 * ((size_t)i * n_atoms + a) + 1] = ff[a].imag();
                }
            }
        }
        if (ms) *ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        write_out(f, d, f_out, d_xyz, d_adp, d_occ);
        return 0;
    } catch (const std::exception &ex) {
        g_last_error = ex.what();
        return 1;
    } catch (...) {
        g_last_error = "unknown exception";
        return 1;
    }
}

// Tabulated path: AnyScatterer engine + ConstFormFactorCalculationsManager with a
// map from Miller index to the per-atom complex form factors.
int ref_table_sf(const double *cell, const char *ops, const char *labels, int n_atoms, const double *xyz, const int *n_adp,
                 const double *adp, const double *occ, const int *mult,
                 int n_keys, const int *keys, const double *values /* [n_keys][n_atoms][2] */,
                 int n_hkl, const int *hkl, const double *dtdf,
                 double *f_out, double *d_xyz, double *d_adp, double *d_occ, double *ms)
{
    try {
        Input in{cell, ops, n_atoms, xyz, n_adp, adp, occ, mult, labels};
        Crystal crystal = make_crystal(in);
        std::map<Vector3i, vector<complex<double> > > table;
        for (int k = 0; k < n_keys; k++) {
            vector<complex<double> > v(n_atoms);
            for (int a = 0; a < n_atoms; a++)
                v[a] = complex<double>(values[2 * ((size_t)k * n_atoms + a)], values[2 * ((size_t)k * n_atoms + a) + 1]);
            table[Vector3i(keys[3 * k], keys[3 * k + 1], keys[3 * k + 2])] = v;
        }
        AnyScattererStructureFactorCalculator calc(crystal);
        std::shared_ptr<AtomicFormFactorCalculationsManager> mgr =
            std::make_shared<ConstFormFactorCalculationsManager>(crystal.unitCell, table);
        calc.setAtomicFormfactorManager(mgr);
        vector<Vector3i> h(n_hkl);
        vector<complex<double> > g(n_hkl), f;
        for (int i = 0; i < n_hkl; i++) {
            h[i] = Vector3i(hkl[3 * i], hkl[3 * i + 1], hkl[3 * i + 2]);
            g[i] = complex<double>(dtdf[2 * i], dtdf[2 * i + 1]);
        }
        vector<bool> inc(n_atoms, true);
        vector<TargetFunctionAtomicParamDerivatives> d;
        auto t0 = std::chrono::steady_clock::now();
        calc.calculateStructureFactorsAndDerivatives(h, f, d, g, inc);
        auto t1 = std::chrono::steady_clock::now();
        if (ms) *ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        write_out(f, d, f_out, d_xyz, d_adp, d_occ);
        return 0;
    } catch (const std::exception &ex) {
        g_last_error = ex.what();
        return 1;
    } catch (...) {
        g_last_error = "unknown exception";
        return 1;
    }
}

// The reference's .tsc reader alone (tsc_io::read_tsc, src/IO/tsc_io.cpp:60-125), timed around the call:
// the scatterer and row counts and the seconds the read took (for the reader comparison in oracle/tsc_speed.py).
int ref_tsc_read(const char *path, int *n_atoms, int *n_rows, double *seconds)
{
    try {
        vector<string> names;
        vector<Vector3i> keys;
        vector<vector<complex<double> > > ff;
        const auto t0 = std::chrono::steady_clock::now();
        tsc_io::read_tsc(path, names, keys, ff);
        *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        *n_atoms = (int)names.size();
        *n_rows = (int)keys.size();
        return 0;
    } catch (const std::exception &ex) {
        g_last_error = ex.what();
        return 1;
    } catch (...) {
        g_last_error = "unknown exception";
        return 1;
    }
}

// The tabulated path from a .tsc file read by the reference's own reader
// (tsc_io::read_tsc, src/IO/tsc_io.cpp:60-125), then as ref_table_sf
// (TscFileBasedSfCalculator, src/Scattering/TscFileBasedSfCalculator.cpp:17-123).
int ref_tsc_sf(const char *path, const double *cell, const char *ops, const char *labels, int n_atoms,
               const double *xyz, const int *n_adp, const double *adp, const double *occ, const int *mult, int n_hkl,
               const int *hkl, const double *dtdf, double *f_out, double *d_xyz, double *d_adp, double *d_occ)
{
    try {
        vector<string> names;
        vector<Vector3i> keys;
        vector<vector<complex<double> > > ff;
        tsc_io::read_tsc(path, names, keys, ff);
        if ((int)names.size() != n_atoms) {
            g_last_error = "tsc file lists a different number of scatterers";
            return 1;
        }
        vector<int> k(3 * keys.size());
        vector<double> v(2 * keys.size() * (size_t)n_atoms);
        for (size_t i = 0; i < keys.size(); i++) {
            for (int j = 0; j < 3; j++) k[3 * i + j] = keys[i][j];
            for (int a = 0; a < n_atoms; a++) {
                v[2 * (i * n_atoms + a)] = ff[i][a].real();
                v[2 * (i * n_atoms + a) + 1] = ff[i][a].imag();
            }
        }
        return ref_table_sf(cell, ops, labels, n_atoms, xyz, n_adp, adp, occ, mult, (int)keys.size(), k.data(),
                            v.data(), n_hkl, hkl, dtdf, f_out, d_xyz, d_adp, d_occ, nullptr);
    } catch (const std::exception &ex) {
        g_last_error = ex.what();
        return 1;
    } catch (...) {
        g_last_error = "unknown exception";
        return 1;
    }
}

// AnyHcCalculator with XD-style local coordinate systems (XdLocalCoordinateSystem, src/HC_Model/
// XdLocalCoordinateSystem.cpp:86-264), the large-molecule implementation and the LCS not frozen
// (src/Scattering/AnyHcCalculator.cpp:117-206): the calculator is built on the atoms at xyz, then
// calculateStructureFactorsAndDerivatives is called with the atoms moved to xyz_moved, so the reference
// recomputes every LCS from the moved geometry (AnyHcCalculator.cpp:236-244, 319-329).
// lcs_def[a] = {central atom, axis 1, axis 2 (+-1..3 for +-X..Z), right-handed, n1, n2a, n2b}: the points
// are sums of the n atoms listed in lcs_atoms (consumed in order) or, with n = 0, the fractional dummy
// position lcs_dummy[a][point][3].  lcs_out: the LCS matrices of the moved geometry [n][3][3] (columns x y z).
int ref_anyhc_lcs(const double *cell, const char *ops, int n_atoms, const double *xyz, const double *xyz_moved,
                  const int *n_adp, const double *adp, const double *occ, const int *mult, const int *atom_wfn,
                  const int *atom_type, const int *lcs_def, const int *lcs_atoms, const double *lcs_dummy,
                  int n_wfn, const int *orb_off, const int *orb_occ, const int *orb_core,
                  const int *sto_off, const int *sto_pow, const double *sto_exp, const double *sto_coeff,
                  const double *def_exp, const int *def_npow, const int *def_pow, const double *wfn_anom,
                  const int *wfn_z, int n_types, const int *type_nl, const double *type_plm, const double *type_pval,
                  const double *type_kappa, const double *type_kappa_p, int n_hkl, const int *hkl,
                  const double *dtdf, int n_threads, double *f_out, double *d_xyz, double *d_adp, double *d_occ,
                  double *lcs_out)
{
    try {
        std::string types;
        vector<string> labels(n_atoms);
        for (int a = 0; a < n_atoms; a++) {
            types += periodic_table::symbol(wfn_z[atom_wfn[a]]) + ";";
            labels[a] = periodic_table::symbol(wfn_z[atom_wfn[a]]) + std::to_string(a + 1);
        }
        Input in{cell, ops, n_atoms, xyz, n_adp, adp, occ, mult, types.c_str()};
        Crystal crystal = make_crystal(in);
        HC_ModelParameters p = make_hc_params(n_atoms, atom_wfn, atom_type, n_wfn, orb_off, orb_occ, orb_core, sto_off,
                                              sto_pow, sto_exp, sto_coeff, def_exp, def_npow, def_pow, wfn_anom, wfn_z,
                                              n_types, type_nl, type_plm, type_pval, type_kappa, type_kappa_p);
        vector<std::shared_ptr<LocalCoordinateSystemInCrystal> > lcs = make_xd_lcs(crystal, labels, n_atoms, lcs_def, lcs_atoms, lcs_dummy);
        AnyHcCalculator calc(crystal, p, lcs, false, false, true, n_threads, false, false, "CPU");
        vector<AtomInCrystal> moved = crystal.atoms;
        for (int a = 0; a < n_atoms; a++)
            moved[a].coordinates = Vector3d(xyz_moved[3 * a], xyz_moved[3 * a + 1], xyz_moved[3 * a + 2]);
        vector<Vector3i> h(n_hkl);
        vector<complex<double> > g(n_hkl), f;
        for (int i = 0; i < n_hkl; i++) {
            h[i] = Vector3i(hkl[3 * i], hkl[3 * i + 1], hkl[3 * i + 2]);
            g[i] = complex<double>(dtdf[2 * i], dtdf[2 * i + 1]);
        }
        vector<TargetFunctionAtomicParamDerivatives> dd;
        calc.calculateStructureFactorsAndDerivatives(moved, h, f, dd, g, vector<bool>(n_atoms, true));
        write_out(f, dd, f_out, d_xyz, d_adp, d_occ);
        Crystal cm = crystal;
        cm.atoms = moved;
        for (int a = 0; a < n_atoms; a++) {
            Matrix3d m;
            lcs[a]->calculate(m, cm);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) lcs_out[9 * a + 3 * i + j] = m(i, j);
        }
        return 0;
    } catch (const std::exception &ex) {
        g_last_error = ex.what();
        return 1;
    } catch (...) {
        g_last_error = "unknown exception";
        return 1;
    }
}

// CombinedStructureFactorCalculator (src/Scattering/CombinedStructureFactorCalculator.cpp:9-52, 124-215) over an
// AnyHcCalculator (XD local coordinate systems as ref_anyhc_lcs, large-molecule implementation) for the atoms in
// hc_atoms and an AnyIamCalculator (the named Gaussian table, src/Scattering/AnyIamCalculator.cpp:13-19) for the
// atoms in iam_atoms, both built on the whole crystal (TAAM's split, HcAtomBankStructureFactorCalculator.cpp:482-499).
// The combined calculator sets every part's anomalous dispersion to zero when it is built (its set()).
int ref_combined_sf(const double *cell, const char *ops, int n_atoms, const double *xyz, const int *n_adp,
                    const double *adp, const double *occ, const int *mult, const int *atom_wfn, const int *atom_type,
                    const int *lcs_def, const int *lcs_atoms, const double *lcs_dummy, int n_hc, const int *hc_atoms,
                    int n_iam, const int *iam_atoms, const char *iam_table,
                    int n_wfn, const int *orb_off, const int *orb_occ, const int *orb_core,
                    const int *sto_off, const int *sto_pow, const double *sto_exp, const double *sto_coeff,
                    const double *def_exp, const int *def_npow, const int *def_pow, const double *wfn_anom,
                    const int *wfn_z, int n_types, const int *type_nl, const double *type_plm,
                    const double *type_pval, const double *type_kappa, const double *type_kappa_p, int n_hkl,
                    const int *hkl, const double *dtdf, double *f_out, double *d_xyz, double *d_adp, double *d_occ)
{
    try {
        std::string types;
        vector<string> labels(n_atoms);
        for (int a = 0; a < n_atoms; a++) {
            types += periodic_table::symbol(wfn_z[atom_wfn[a]]) + ";";
            labels[a] = periodic_table::symbol(wfn_z[atom_wfn[a]]) + std::to_string(a + 1);
        }
        Input in{cell, ops, n_atoms, xyz, n_adp, adp, occ, mult, types.c_str()};
        Crystal crystal = make_crystal(in);
        HC_ModelParameters p = make_hc_params(n_atoms, atom_wfn, atom_type, n_wfn, orb_off, orb_occ, orb_core, sto_off,
                                              sto_pow, sto_exp, sto_coeff, def_exp, def_npow, def_pow, wfn_anom, wfn_z,
                                              n_types, type_nl, type_plm, type_pval, type_kappa, type_kappa_p);
        vector<std::shared_ptr<LocalCoordinateSystemInCrystal> > lcs =
            make_xd_lcs(crystal, labels, n_atoms, lcs_def, lcs_atoms, lcs_dummy);
        vector<std::shared_ptr<SfCalculator> > calcs{
            std::make_shared<AnyHcCalculator>(crystal, p, lcs, false, false, true, 1, false, false, "CPU"),
            std::make_shared<AnyIamCalculator>(crystal, false, string(iam_table))};
        vector<vector<int> > parts{vector<int>(hc_atoms, hc_atoms + n_hc), vector<int>(iam_atoms, iam_atoms + n_iam)};
        CombinedStructureFactorCalculator calc(calcs, parts);
        vector<Vector3i> h(n_hkl);
        vector<complex<double> > g(n_hkl), f;
        for (int i = 0; i < n_hkl; i++) {
            h[i] = Vector3i(hkl[3 * i], hkl[3 * i + 1], hkl[3 * i + 2]);
            g[i] = complex<double>(dtdf[2 * i], dtdf[2 * i + 1]);
        }
        vector<TargetFunctionAtomicParamDerivatives> dd;
        calc.calculateStructureFactorsAndDerivatives(crystal.atoms, h, f, dd, g, vector<bool>(n_atoms, true));
        write_out(f, dd, f_out, d_xyz, d_adp, d_occ);
        return 0;
    } catch (const std::exception &ex) {
        g_last_error = ex.what();
        return 1;
    } catch (...) {
        g_last_error = "unknown exception";
        return 1;
    }
}

} // extern "C"
