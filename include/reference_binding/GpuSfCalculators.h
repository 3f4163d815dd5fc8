/* Reference-side binding: DiSCaMB SfCalculator subclasses that run on the GB300 engine.
 *
 * This header belongs to a DiSCaMB build (it includes DiSCaMB's own headers) and is what a maintainer adds to the
 * reference to use the engine as a drop-in.  It converts the reference's types into the C ABI descriptors of
 * dsf_gb300.h and delegates to the C++ layer of dsf_calculator.hpp:
 *
 *   GpuHcCalculator       AnyHcCalculator / HansenCoppensStructureFactorCalculator
 *                         (src/Scattering/AnyHcCalculator.cpp:13-26, 117-206, 218-329;
 *                          src/Scattering/HansenCoppensStructureFactorCalculator.cpp:57-72, 107-290, 380-508),
 *                         local coordinate systems recomputed on every update unless frozen
 *   GpuIamCalculator      AnyIamCalculator (src/Scattering/AnyIamCalculator.cpp:13-154)
 *   createGpuSfCalculator the factory branch SfCalculator::create would take for the model names
 *                         "hc_gb300", "iam_gb300" (src/Scattering/SfCalculator.cpp:343-385)
 *
 * TAAM's split (CombinedStructureFactorCalculator over an HC and an IAM calculator,
 * HcAtomBankStructureFactorCalculator.cpp:482-520) works unchanged with these as its parts; dsf::CombinedCalculator
 * in dsf_calculator.hpp is the same split with the parts in one batched submission.
 *
 * Link with libdsf_gb300.so; include paths: DiSCaMB's include/ and third-party/ (json.hpp), and this
 * repository's include/.
 */
#pragma once

#include "discamb/BasicUtilities/on_error.h"
#include "discamb/CrystalStructure/Crystal.h"
#include "discamb/CrystalStructure/LocalCoordinateSystemInCrystal.h"
#include "discamb/HC_Model/HC_ModelParameters.h"
#include "discamb/Scattering/NGaussianFormFactorsTable.h"
#include "discamb/Scattering/SfCalculator.h"

#include "../dsf_calculator.hpp"

#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace discamb {
namespace gb300 {

// the dsf_symmetry of a crystal, with the arrays it points to
struct SymmetryDesc {
    std::vector<int> rot;
    std::vector<double> trans;
    dsf_symmetry sym{};
};

// engine = true: the HC CPU engine's representation (the subset of operations modulo inversion and centering,
// the inversion handled by the engine, HansenCoppensStructureFactorCalculator.cpp:107-155); false: every
// operation modulo centering (the generic engine, AnyScattererStructureFactorCalculator.cpp:40-66).  Centering
// enters as the per-reflection multiplier in both.
inline void makeSymmetry(const Crystal &crystal, bool engine, SymmetryDesc &d)
{
    const SpaceGroup &sg = crystal.spaceGroup;
    const int n_sub = sg.nSymmetryOperationsInSubset();
    const bool centro = sg.isCentrosymmetric();
    d.rot.clear();
    d.trans.clear();
    for (int inv = 0; inv < ((!engine && centro) ? 2 : 1); inv++)
        for (int i = 0; i < n_sub; i++) {
            Matrix3<int> r;
            Vector3d t;
            sg.getSpaceGroupOperation(0, inv, i).getRotation(r);
            sg.getSpaceGroupOperation(0, inv, i).getTranslation(t);
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) d.rot.push_back(r(a, b));
            for (int a = 0; a < 3; a++) d.trans.push_back(t[a]);
        }
    dsf_symmetry &s = d.sym;
    s.cell[0] = crystal.unitCell.a();
    s.cell[1] = crystal.unitCell.b();
    s.cell[2] = crystal.unitCell.c();
    s.cell[3] = crystal.unitCell.alpha();
    s.cell[4] = crystal.unitCell.beta();
    s.cell[5] = crystal.unitCell.gamma();
    s.n_symops = (int)d.rot.size() / 9;
    s.symop_rotation = d.rot.data();
    s.symop_translation = d.trans.data();
    s.centrosymmetric = (engine && centro) ? 1 : 0;
    if (engine && centro) {
        Vector3<CrystallographicRational> t;
        sg.inversionCenterTranslation(t);
        for (int a = 0; a < 3; a++) s.inversion_translation[a] = t[a].get();
    }
    bool obverse = true;
    s.centering = sg.centering(obverse);
    s.obverse = obverse ? 1 : 0;
    s.n_symops_total = sg.nSymmetryOperations();
}

// the spherical densities of a wavefunction type as density terms c r^n exp(-z r): the orbital products summed
// with their occupancies, as sto_atomic_wfn::atomicStoWfnToSphericalDensity (src/HC_Model/HC_WfnData.cpp:11-70);
// the valence density normalised to one electron, as setModel does
// (HansenCoppensStructureFactorCalculator.cpp:187-218)
inline void densityTerms(const HC_WfnType &w, bool core, std::vector<double> &c, std::vector<double> &z,
                         std::vector<int> &n)
{
    const std::vector<int> &idx = core ? w.core_orbitals_indices : w.valence_orbitals_indices;
    const size_t first = c.size();
    double electrons = 0;
    for (int k : idx) {
        const double occ = w.orbital_occupancy[k];
        electrons += occ;
        if (occ == 0) continue;
        const SlaterTypeAtomicOrbitalRdf &o = w.orbitals[k];
        for (size_t i = 0; i < o.coefficients.size(); i++)
            for (size_t j = 0; j <= i; j++) {
                c.push_back(o.coefficients[i] * o.coefficients[j] * occ / (4.0 * M_PI) * (i == j ? 1.0 : 2.0));
                z.push_back(o.exponents[i] + o.exponents[j]);
                n.push_back(o.power_r[i] + o.power_r[j]);
            }
    }
    if (!core && electrons != 0)
        for (size_t q = first; q < c.size(); q++) c[q] /= electrons;
}

// the dsf_hc_model of HC_ModelParameters, with the arrays it points to
struct HcModelDesc {
    std::vector<int> core_off{0}, core_pow, val_off{0}, val_pow, def_npow, def_pow, type_nl;
    std::vector<double> core_c, core_z, val_c, val_z, def_exp, anom, plm, pval, kappa, kappa_p;
    dsf_hc_model model{};
};

inline void makeHcModel(const HC_ModelParameters &p, HcModelDesc &d)
{
    for (const HC_WfnType &w : p.wfn_parameters) {
        densityTerms(w, true, d.core_c, d.core_z, d.core_pow);
        d.core_off.push_back((int)d.core_c.size());
        densityTerms(w, false, d.val_c, d.val_z, d.val_pow);
        d.val_off.push_back((int)d.val_c.size());
        d.def_exp.push_back(w.deformation_valence_exponent);
        const int np = (int)std::min<size_t>(5, w.deformation_valence_power.size());
        d.def_npow.push_back(np);
        for (int l = 0; l < 5; l++) d.def_pow.push_back(l < np ? w.deformation_valence_power[l] : 0);
        d.anom.push_back(w.anomalous_scattering.real());
        d.anom.push_back(w.anomalous_scattering.imag());
    }
    for (const HC_AtomTypeParameters &t : p.type_parameters) {
        d.type_nl.push_back((int)t.p_lm.size());
        std::vector<double> q(25, 0.0);
        for (size_t l = 0; l < t.p_lm.size() && l < 5; l++)
            for (size_t m = 0; m < t.p_lm[l].size() && m < 2 * l + 1; m++) q[l * l + m] = t.p_lm[l][m];
        d.plm.insert(d.plm.end(), q.begin(), q.end());
        d.pval.push_back(t.p_val);
        d.kappa.push_back(t.kappa_spherical_valence);
        d.kappa_p.push_back(t.kappa_deformation_valence);
    }
    // never-read sentinels keep every pointer valid for models without terms of a kind
    for (auto *v : {&d.core_c, &d.val_c}) v->push_back(0.0);
    for (auto *v : {&d.core_z, &d.val_z}) v->push_back(1.0);
    for (auto *v : {&d.core_pow, &d.val_pow}) v->push_back(0);
    dsf_hc_model &m = d.model;
    m.n_wfn = (int)p.wfn_parameters.size();
    m.core_offset = d.core_off.data();
    m.core_coeff = d.core_c.data();
    m.core_exp = d.core_z.data();
    m.core_pow = d.core_pow.data();
    m.val_offset = d.val_off.data();
    m.val_coeff = d.val_c.data();
    m.val_exp = d.val_z.data();
    m.val_pow = d.val_pow.data();
    m.def_val_exp = d.def_exp.data();
    m.def_val_npow = d.def_npow.data();
    m.def_val_pow = d.def_pow.data();
    m.anomalous = d.anom.data();
    m.n_types = (int)p.type_parameters.size();
    m.type_nl = d.type_nl.data();
    m.type_plm = d.plm.data();
    m.type_pval = d.pval.data();
    m.type_kappa = d.kappa.data();
    m.type_kappa_prime = d.kappa_p.data();
}

// the dsf_atoms of a crystal's atoms, with the arrays it points to
struct AtomsDesc {
    std::vector<int> wfn, type, nadp;
    std::vector<double> lcs, mult;
    dsf_atoms atoms{};
};

inline void makeAtoms(const Crystal &crystal, const std::vector<int> &wfn, const std::vector<int> &type,
                      const std::vector<double> &lcs, AtomsDesc &d)
{
    const size_t n = crystal.atoms.size();
    d.wfn = wfn.empty() ? std::vector<int>(n, 0) : wfn;
    d.type = type;
    d.lcs = lcs;
    d.nadp.resize(n);
    d.mult.resize(n);
    for (size_t a = 0; a < n; a++) {
        d.nadp[a] = (int)crystal.atoms[a].adp.size();
        d.mult[a] = crystal.atoms[a].multiplicity;
    }
    dsf_atoms &t = d.atoms;
    t.n_atoms = (int)n;
    t.atom_wfn = d.wfn.data();
    t.atom_type = d.type.data();
    t.adp_components = d.nadp.data();
    t.lcs = d.lcs.empty() ? nullptr : d.lcs.data();
    t.multiplicity = d.mult.data();
    t.anomalous = nullptr;
    t.xyz_convention = crystal.xyzCoordinateSystem == structural_parameters_convention::XyzCoordinateSystem::cartesian
                           ? DSF_XYZ_CARTESIAN : DSF_XYZ_FRACTIONAL;
    t.adp_convention = crystal.adpConvention == structural_parameters_convention::AdpConvention::U_cart ? DSF_ADP_U_CART
                       : crystal.adpConvention == structural_parameters_convention::AdpConvention::U_star
                           ? DSF_ADP_U_STAR : DSF_ADP_U_CIF;
}

inline std::vector<dsf::AtomInCrystal> toEngine(const std::vector<AtomInCrystal> &atoms)
{
    std::vector<dsf::AtomInCrystal> out(atoms.size());
    for (size_t a = 0; a < atoms.size(); a++) {
        for (int k = 0; k < 3; k++) out[a].coordinates[k] = atoms[a].coordinates[k];
        out[a].adp = atoms[a].adp;
        out[a].occupancy = atoms[a].occupancy;
    }
    return out;
}

inline std::vector<dsf::Vector3i> toEngine(const std::vector<Vector3i> &hkl)
{
    std::vector<dsf::Vector3i> out(hkl.size());
    for (size_t i = 0; i < hkl.size(); i++) out[i] = {hkl[i][0], hkl[i][1], hkl[i][2]};
    return out;
}

inline void fromEngine(const std::vector<dsf::TargetFunctionAtomicParamDerivatives> &in,
                       std::vector<TargetFunctionAtomicParamDerivatives> &out)
{
    out.resize(in.size());
    for (size_t a = 0; a < in.size(); a++) {
        for (int k = 0; k < 3; k++) out[a].atomic_position_derivatives[k] = in[a].atomic_position_derivatives[k];
        out[a].adp_derivatives = in[a].adp_derivatives;
        out[a].occupancy_derivatives = in[a].occupancy_derivatives;
    }
}

inline dsf::DerivativesSelector toEngine(const DerivativesSelector &s)
{
    dsf::DerivativesSelector d;
    d.d_xyz = s.d_xyz;
    d.d_adp = s.d_adp;
    d.d_occ = s.d_occ;
    d.d_anom = s.d_anom;
    return d;
}

// one engine per device for the whole process, shared by the calculators
inline std::shared_ptr<dsf::Engine> engineFor(int device)
{
    static std::map<int, std::weak_ptr<dsf::Engine> > engines;
    std::shared_ptr<dsf::Engine> e = engines[device].lock();
    if (!e) {
        e = std::make_shared<dsf::Engine>(device);
        engines[device] = e;
    }
    return e;
}

// the engine's errors become the reference's exceptions (on_error.h:24-36)
template <typename F>
void guarded(F &&f)
{
    try {
        f();
    } catch (const dsf::Error &e) {
        on_error::throwException(e.what(), __FILE__, __LINE__);
    }
}

// calls shared by the two calculators: the reference's SfCalculator interface over a dsf::SfCalculator
class GpuSfCalculatorBase : public SfCalculator {
public:
    void setAnomalous(const std::vector<std::complex<double> > &anomalous) override
    {
        guarded([&] { mCalc->setAnomalous(anomalous); });
    }
    void calculateStructureFactorsAndDerivatives(const std::vector<AtomInCrystal> &atoms,
                                                 const std::vector<Vector3i> &hkl,
                                                 std::vector<std::complex<double> > &f,
                                                 std::vector<TargetFunctionAtomicParamDerivatives> &dTarget_dparam,
                                                 const std::vector<std::complex<double> > &dTarget_df,
                                                 const std::vector<bool> &countAtomContribution) override
    {
        std::vector<dsf::TargetFunctionAtomicParamDerivatives> d;
        guarded([&] {
            mCalc->calculateStructureFactorsAndDerivatives(toEngine(atoms), toEngine(hkl), f, d, dTarget_df,
                                                           countAtomContribution);
        });
        fromEngine(d, dTarget_dparam);
    }
    void calculateStructureFactorsAndDerivatives(const std::vector<AtomInCrystal> &atoms,
                                                 const std::vector<Vector3i> &hkl,
                                                 std::vector<std::complex<double> > &f,
                                                 std::vector<TargetFunctionAtomicParamDerivatives> &dTarget_dparam,
                                                 const std::vector<std::complex<double> > &dTarget_df,
                                                 const std::vector<bool> &countAtomContribution,
                                                 const DerivativesSelector &selector) override
    {
        std::vector<dsf::TargetFunctionAtomicParamDerivatives> d;
        guarded([&] {
            mCalc->calculateStructureFactorsAndDerivatives(toEngine(atoms), toEngine(hkl), f, d, dTarget_df,
                                                           countAtomContribution, toEngine(selector));
        });
        fromEngine(d, dTarget_dparam);
    }
    void calculateStructureFactors(const std::vector<AtomInCrystal> &atoms, const std::vector<Vector3i> &hkl,
                                   std::vector<std::complex<double> > &f,
                                   const std::vector<bool> &countAtomContribution) override
    {
        guarded([&] { mCalc->calculateStructureFactors(toEngine(atoms), toEngine(hkl), f, countAtomContribution); });
    }
    void update(const std::vector<AtomInCrystal> &atoms) override
    {
        guarded([&] { mCalc->update(toEngine(atoms)); });
    }
    void calculateStructureFactorsAndDerivatives(const Vector3i &hkl, std::complex<double> &scatteringFactor,
                                                 SfDerivativesAtHkl &derivatives,
                                                 const std::vector<bool> &countAtomContribution) override
    {
        dsf::SfDerivativesAtHkl d;
        guarded([&] {
            mCalc->calculateStructureFactorsAndDerivatives(dsf::Vector3i{hkl[0], hkl[1], hkl[2]}, scatteringFactor, d,
                                                           countAtomContribution);
        });
        const size_t n = d.occupancyDerivatives.size();
        derivatives.atomicPostionDerivatives.resize(n);
        for (size_t a = 0; a < n; a++)
            for (int k = 0; k < 3; k++) derivatives.atomicPostionDerivatives[a][k] = d.atomicPostionDerivatives[a][k];
        derivatives.adpDerivatives = d.adpDerivatives;
        derivatives.occupancyDerivatives = d.occupancyDerivatives;
        derivatives.anomalousScatteringDerivatives.clear();  // f', f'' are inputs here
    }
    void calculateFormFactors(const Vector3i &hkl, std::vector<std::complex<double> > &formFactors,
                              const std::vector<bool> &includeAtom) const override
    {
        guarded([&] { mCalc->calculateFormFactors(dsf::Vector3i{hkl[0], hkl[1], hkl[2]}, formFactors, includeAtom); });
    }
    void getModelInformation(std::vector<std::pair<std::string, std::string> > &modelInfo) const override
    {
        mCalc->getModelInformation(modelInfo);
    }
    std::string name() const override { return mCalc->name(); }
    // "precision": "fp64" (the reference's, default) or "fp32" (FP32 bulk sums, FP64 accumulation)
    void setPrecision(const std::string &p) { mCalc->setPrecision(p == "fp32" ? DSF_FP32_BULK : DSF_FP64); }

protected:
    std::shared_ptr<dsf::SfCalculator> mCalc;
};

// AnyHcCalculator on the GB300 engine (model "hc_gb300").  The local coordinate systems are the reference's own
// objects: they are computed at construction and, unless frozenLcs, again from the atoms of every update and every
// calculation, and the engine gets the new matrices (AnyHcCalculator.cpp:236-244, 319-329).
class GpuHcCalculator : public GpuSfCalculatorBase {
public:
    GpuHcCalculator(const Crystal &crystal, const HC_ModelParameters &parameters,
                    const std::vector<std::shared_ptr<LocalCoordinateSystemInCrystal> > &lcs, bool frozenLcs = false,
                    int device = 0)
        : mCrystal(crystal), mLcs(lcs), mFrozen(frozenLcs)
    {
        SymmetryDesc sym;
        makeSymmetry(crystal, true, sym);
        HcModelDesc model;
        makeHcModel(parameters, model);
        AtomsDesc atoms;
        makeAtoms(crystal, parameters.atom_to_wfn_map, parameters.atom_to_type_map, lcsMatrices(crystal.atoms), atoms);
        guarded([&] { mHc = std::make_shared<dsf::HcCalculator>(engineFor(device), sym.sym, model.model, atoms.atoms); });
        mCalc = mHc;
        mCalc->update(toEngine(crystal.atoms));
        mLast = atoms.lcs;
    }
    void update(const std::vector<AtomInCrystal> &atoms) override
    {
        refreshLcs(atoms);
        GpuSfCalculatorBase::update(atoms);
    }
    void calculateStructureFactorsAndDerivatives(const std::vector<AtomInCrystal> &atoms,
                                                 const std::vector<Vector3i> &hkl,
                                                 std::vector<std::complex<double> > &f,
                                                 std::vector<TargetFunctionAtomicParamDerivatives> &dTarget_dparam,
                                                 const std::vector<std::complex<double> > &dTarget_df,
                                                 const std::vector<bool> &countAtomContribution) override
    {
        refreshLcs(atoms);
        GpuSfCalculatorBase::calculateStructureFactorsAndDerivatives(atoms, hkl, f, dTarget_dparam, dTarget_df,
                                                                     countAtomContribution);
    }
    void calculateStructureFactorsAndDerivatives(const std::vector<AtomInCrystal> &atoms,
                                                 const std::vector<Vector3i> &hkl,
                                                 std::vector<std::complex<double> > &f,
                                                 std::vector<TargetFunctionAtomicParamDerivatives> &dTarget_dparam,
                                                 const std::vector<std::complex<double> > &dTarget_df,
                                                 const std::vector<bool> &countAtomContribution,
                                                 const DerivativesSelector &selector) override
    {
        refreshLcs(atoms);
        GpuSfCalculatorBase::calculateStructureFactorsAndDerivatives(atoms, hkl, f, dTarget_dparam, dTarget_df,
                                                                     countAtomContribution, selector);
    }
    void calculateStructureFactors(const std::vector<AtomInCrystal> &atoms, const std::vector<Vector3i> &hkl,
                                   std::vector<std::complex<double> > &f,
                                   const std::vector<bool> &countAtomContribution) override
    {
        refreshLcs(atoms);
        GpuSfCalculatorBase::calculateStructureFactors(atoms, hkl, f, countAtomContribution);
    }
    void setElectronScattering(bool on, const std::vector<int> &wfn_z, const std::vector<double> &wfn_f000)
    {
        guarded([&] { mHc->setElectronScattering(on, wfn_z, wfn_f000); });
    }

private:
    Crystal mCrystal;
    std::vector<std::shared_ptr<LocalCoordinateSystemInCrystal> > mLcs;
    bool mFrozen;
    std::shared_ptr<dsf::HcCalculator> mHc;
    std::vector<double> mLast;

    // row-major [n][3][3], columns = local x, y, z (LocalCoordinateSystemInCrystal::calculate's matrix)
    std::vector<double> lcsMatrices(const std::vector<AtomInCrystal> &atoms)
    {
        if (mLcs.empty()) return {};
        Crystal c = mCrystal;
        c.atoms = atoms;
        std::vector<double> out(9 * mLcs.size());
        for (size_t a = 0; a < mLcs.size(); a++) {
            Matrix3d m;
            mLcs[a]->calculate(m, c);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) out[9 * a + 3 * i + j] = m(i, j);
        }
        return out;
    }
    void refreshLcs(const std::vector<AtomInCrystal> &atoms)
    {
        if (mFrozen || mLcs.empty()) return;
        std::vector<double> m = lcsMatrices(atoms);
        if (m == mLast) return;
        guarded([&] { mHc->engine()->check(dsf_structure_set_lcs(mHc->structure(), m.data()), "set_lcs"); });
        mLast.swap(m);
    }
};

// AnyIamCalculator on the GB300 engine (model "iam_gb300"): n-Gaussian form factors of the atom type labels from
// the named table (NGaussianFormFactorsTable), every operation modulo centering
class GpuIamCalculator : public GpuSfCalculatorBase {
public:
    GpuIamCalculator(const Crystal &crystal, const std::string &table = "IT92", int device = 0)
    {
        SymmetryDesc sym;
        makeSymmetry(crystal, false, sym);
        std::vector<std::string> labels;
        std::vector<int> type(crystal.atoms.size());
        for (size_t a = 0; a < crystal.atoms.size(); a++) {
            auto it = std::find(labels.begin(), labels.end(), crystal.atoms[a].type);
            type[a] = (int)(it - labels.begin());
            if (it == labels.end()) labels.push_back(crystal.atoms[a].type);
        }
        std::vector<int> ng(labels.size());
        std::vector<double> ga(5 * labels.size(), 0.0), gb(5 * labels.size(), 0.0), gc(labels.size());
        for (size_t t = 0; t < labels.size(); t++) {
            std::vector<double> a, b;
            n_gaussian_form_factors_table::getFormFactor(labels[t], table).get_parameters(a, b, gc[t]);
            ng[t] = (int)std::min<size_t>(5, a.size());
            for (int q = 0; q < ng[t]; q++) {
                ga[5 * t + q] = a[q];
                gb[5 * t + q] = b[q];
            }
        }
        dsf_iam_model model{(int)labels.size(), ng.data(), ga.data(), gb.data(), gc.data()};
        AtomsDesc atoms;
        makeAtoms(crystal, {}, type, {}, atoms);
        guarded([&] {
            mCalc = std::make_shared<dsf::IamCalculator>(engineFor(device), sym.sym, model, atoms.atoms, table);
        });
        mCalc->update(toEngine(crystal.atoms));
    }
};

// The factory branch for the engine's model names (SfCalculator::create, src/Scattering/SfCalculator.cpp:343-385);
// null for other names.  "hc_gb300" needs the HC model and local coordinate systems, which the reference reads from
// its model files before it builds an AnyHcCalculator; they are passed here the same way.
inline SfCalculator *createGpuSfCalculator(const Crystal &crystal, const std::string &modelName,
                                           const nlohmann::json &details, const HC_ModelParameters *hc = nullptr,
                                           const std::vector<std::shared_ptr<LocalCoordinateSystemInCrystal> > *lcs =
                                               nullptr)
{
    const int device = details.value("device", 0);
    const std::string precision = details.value("precision", std::string("fp64"));
    GpuSfCalculatorBase *c = nullptr;
    if (modelName == "iam_gb300")
        c = new GpuIamCalculator(crystal, details.value("table", std::string("IT92")), device);
    else if (modelName == "hc_gb300") {
        if (!hc || !lcs) on_error::throwException("hc_gb300 needs the HC model and the LCS", __FILE__, __LINE__);
        c = new GpuHcCalculator(crystal, *hc, *lcs, details.value("frozen lcs", false), device);
    }
    if (c) c->setPrecision(precision);
    return c;
}

}  // namespace gb300
}  // namespace discamb
