/* C++ host layer over the dsf_gb300 C ABI, with the calls and argument
 * meaning of the reference's SfCalculator (include/discamb/Scattering/
 * SfCalculator.h:20-122):
 *
 *   calculateStructureFactorsAndDerivatives(atoms, hkl, f, dTarget_dparam,
 *       dTarget_df, countAtomContribution)          SfCalculator.h:45-67
 *   the same without countAtomContribution, and with a DerivativesSelector
 *   calculateStructureFactors(atoms, hkl, f, countAtomContribution)
 *   calculateStructureFactorsAndDerivatives(hkl, f, SfDerivativesAtHkl,
 *       countAtomContribution)    (single h)        SfCalculator.h:82-86
 *   calculateFormFactors(hkl, ff, includeAtom)      SfCalculator.h:89
 *   update(atoms), setAnomalous(anomalous), setN_threads(n), getModelInformation(info), name()
 *
 * The reflection set stays resident on the GPU between calls (it is re-sent
 * only when the caller passes another one), the atoms' parameters travel with
 * every call.  Errors throw dsf::Error with the engine's message, where the
 * reference throws discamb::Exception (on_error.h:24-36).  Header only; link
 * with libdsf_gb300.so.  The types mirror the fields of the reference's
 * AtomInCrystal, TargetFunctionAtomicParamDerivatives and SfDerivativesAtHkl
 * (SF_CalcDataTypes.h:36-64) that the path reads and writes; a shim in the
 * reference (a SfCalculator subclass) converts its own types into these.
 */
#pragma once

#include "dsf_gb300.h"

#include <array>
#include <complex>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace dsf {

using Vector3i = std::array<int, 3>;
using Vector3d = std::array<double, 3>;
using cplx = std::complex<double>;

struct AtomInCrystal {
    Vector3d coordinates{};   // in the crystal's xyz convention (fractional by default)
    std::vector<double> adp;  // 0, 1 (U_iso) or 6 components, in the crystal's ADP convention
    double occupancy = 1.0;
};

struct TargetFunctionAtomicParamDerivatives {
    Vector3d atomic_position_derivatives{};
    std::vector<double> adp_derivatives;
    double occupancy_derivatives = 0.0;
};

struct SfDerivativesAtHkl {
    std::vector<std::array<cplx, 3> > atomicPostionDerivatives;  // the reference's spelling
    std::vector<std::vector<cplx> > adpDerivatives;
    std::vector<cplx> occupancyDerivatives;
};

// SF_CalcDataTypes.h:22-27; d_anom has no counterpart (the engine takes f', f'' as inputs)
struct DerivativesSelector {
    bool d_xyz = true;
    bool d_adp = true;
    bool d_occ = true;
    bool d_anom = true;
};

class Error : public std::runtime_error {
public:
    using std::runtime_error::runtime_error;
};

// one GPU and its stream
class Engine {
public:
    explicit Engine(int device = 0)
    {
        if (dsf_engine_create(device, &e_) != DSF_OK) throw Error("dsf_engine_create failed");
    }
    ~Engine() { dsf_engine_destroy(e_); }
    Engine(const Engine &) = delete;
    Engine &operator=(const Engine &) = delete;
    dsf_engine *get() const { return e_; }
    void check(int rc, const char *what) const
    {
        if (rc != DSF_OK) throw Error(std::string(what) + ": " + dsf_last_error(e_));
    }

private:
    dsf_engine *e_ = nullptr;
};

class SfCalculator {
public:
    virtual ~SfCalculator() { dsf_structure_destroy(s_); }
    SfCalculator(const SfCalculator &) = delete;
    SfCalculator &operator=(const SfCalculator &) = delete;

    // DSF_FP64 (the reference's precision, default) or DSF_FP32_BULK
    void setPrecision(int precision) { precision_ = precision; }
    // the engine threads itself; kept so callers that set it run unchanged
    void setN_threads(int) {}

    void calculateStructureFactorsAndDerivatives(const std::vector<AtomInCrystal> &atoms,
                                                 const std::vector<Vector3i> &hkl, std::vector<cplx> &f,
                                                 std::vector<TargetFunctionAtomicParamDerivatives> &dTarget_dparam,
                                                 const std::vector<cplx> &dTarget_df,
                                                 const std::vector<bool> &countAtomContribution)
    {
        if (dTarget_df.size() != hkl.size()) throw Error("dTarget_df and hkl sizes differ");
        run(atoms, hkl, dTarget_df, countAtomContribution, DSF_D_XYZ | DSF_D_ADP | DSF_D_OCC, f, &dTarget_dparam);
    }

    // every atom counted (SfCalculator.h:52-57)
    void calculateStructureFactorsAndDerivatives(const std::vector<AtomInCrystal> &atoms,
                                                 const std::vector<Vector3i> &hkl, std::vector<cplx> &f,
                                                 std::vector<TargetFunctionAtomicParamDerivatives> &dTarget_dparam,
                                                 const std::vector<cplx> &dTarget_df)
    {
        calculateStructureFactorsAndDerivatives(atoms, hkl, f, dTarget_dparam, dTarget_df, std::vector<bool>());
    }

    // only the selected derivative classes are computed; the others come back zero (SfCalculator.h:59-66, whose
    // default computes them all)
    void calculateStructureFactorsAndDerivatives(const std::vector<AtomInCrystal> &atoms,
                                                 const std::vector<Vector3i> &hkl, std::vector<cplx> &f,
                                                 std::vector<TargetFunctionAtomicParamDerivatives> &dTarget_dparam,
                                                 const std::vector<cplx> &dTarget_df,
                                                 const std::vector<bool> &countAtomContribution,
                                                 const DerivativesSelector &selector)
    {
        if (dTarget_df.size() != hkl.size()) throw Error("dTarget_df and hkl sizes differ");
        const int flags = (selector.d_xyz ? DSF_D_XYZ : 0) | (selector.d_adp ? DSF_D_ADP : 0) |
                          (selector.d_occ ? DSF_D_OCC : 0);
        run(atoms, hkl, dTarget_df, countAtomContribution, flags, f, &dTarget_dparam);
    }

    void calculateStructureFactors(const std::vector<AtomInCrystal> &atoms, const std::vector<Vector3i> &hkl,
                                   std::vector<cplx> &f, const std::vector<bool> &countAtomContribution)
    {
        run(atoms, hkl, std::vector<cplx>(hkl.size(), cplx(1.0, 0.0)), countAtomContribution, 0, f, nullptr);
    }

    // the atoms of the following single-h and form-factor calls
    void update(const std::vector<AtomInCrystal> &atoms) { atoms_ = atoms; }

    // per-atom anomalous dispersion f' + i f'' (SfCalculator::setAnomalous)
    void setAnomalous(const std::vector<cplx> &anomalous)
    {
        if (anomalous.size() != (size_t)n_atoms_) throw Error("anomalous dispersion size differs from the atom count");
        engine_->check(dsf_structure_set_anomalous(s_, reinterpret_cast<const double *>(anomalous.data())),
                       "setAnomalous");
    }

    // F and dF/dparam at one reflection, with the atoms of the last call or update: two one-reflection calls
    // (dT/dF = 1 gives dA/dp, dT/dF = i gives dB/dp); the resident reflection set is restored afterwards
    void calculateStructureFactorsAndDerivatives(const Vector3i &hkl, cplx &f, SfDerivativesAtHkl &d,
                                                 const std::vector<bool> &countAtomContribution)
    {
        if (atoms_.empty()) throw Error("no atoms: call update() or a whole-set calculation first");
        const std::vector<Vector3i> keep = hkl_;
        std::vector<cplx> fa, fb;
        std::vector<TargetFunctionAtomicParamDerivatives> da, db;
        try {
            run(atoms_, {hkl}, {cplx(1.0, 0.0)}, countAtomContribution, DSF_D_XYZ | DSF_D_ADP | DSF_D_OCC, fa, &da);
            run(atoms_, {hkl}, {cplx(0.0, 1.0)}, countAtomContribution, DSF_D_XYZ | DSF_D_ADP | DSF_D_OCC, fb, &db);
        } catch (...) {
            restore(keep);
            throw;
        }
        restore(keep);
        f = fa[0];
        const size_t n = da.size();
        d.atomicPostionDerivatives.resize(n);
        d.adpDerivatives.resize(n);
        d.occupancyDerivatives.resize(n);
        for (size_t a = 0; a < n; a++) {
            for (int k = 0; k < 3; k++)
                d.atomicPostionDerivatives[a][k] = cplx(da[a].atomic_position_derivatives[k], db[a].atomic_position_derivatives[k]);
            d.adpDerivatives[a].resize(da[a].adp_derivatives.size());
            for (size_t k = 0; k < da[a].adp_derivatives.size(); k++)
                d.adpDerivatives[a][k] = cplx(da[a].adp_derivatives[k], db[a].adp_derivatives[k]);
            d.occupancyDerivatives[a] = cplx(da[a].occupancy_derivatives, db[a].occupancy_derivatives);
        }
    }

    // form factors of every atom at one reflection (no anomalous dispersion; HC and IAM)
    void calculateFormFactors(const Vector3i &hkl, std::vector<cplx> &ff, const std::vector<bool> &includeAtom) const
    {
        std::vector<int> inc(includeAtom.begin(), includeAtom.end());
        ff.assign((size_t)n_atoms_, cplx(0.0, 0.0));
        engine_->check(dsf_form_factors(s_, hkl.data(), inc.empty() ? nullptr : inc.data(),
                                        reinterpret_cast<double *>(ff.data())),
                       "calculateFormFactors");
    }

    // (key, value) pairs describing the model (SfCalculator::getModelInformation, SfCalculator.h:41)
    virtual void getModelInformation(std::vector<std::pair<std::string, std::string> > &modelInfo) const
    {
        modelInfo.clear();
    }
    virtual std::string name() const { return "undefined"; }

    int64_t deviceBytes() const { return dsf_structure_device_bytes(s_); }
    dsf_structure *structure() const { return s_; }

protected:
    SfCalculator(std::shared_ptr<Engine> engine, const dsf_atoms &atoms) : engine_(std::move(engine)), n_atoms_(atoms.n_atoms)
    {
        nadp_.assign(atoms.adp_components, atoms.adp_components + atoms.n_atoms);
    }
    std::shared_ptr<Engine> engine_;
    dsf_structure *s_ = nullptr;
    std::vector<Vector3i> hkl_;
    bool have_hkl_ = false;

    void setHkl(const std::vector<Vector3i> &hkl)
    {
        engine_->check(dsf_structure_set_hkl(s_, (int)hkl.size(), hkl.empty() ? nullptr : hkl[0].data()), "set_hkl");
        hkl_ = hkl;
        have_hkl_ = true;
    }

private:
    int n_atoms_ = 0;
    std::vector<int> nadp_;
    int precision_ = DSF_FP64;
    std::vector<AtomInCrystal> atoms_;

    void restore(const std::vector<Vector3i> &keep)
    {
        if (keep != hkl_) setHkl(keep);
    }

    void run(const std::vector<AtomInCrystal> &atoms, const std::vector<Vector3i> &hkl, const std::vector<cplx> &dtdf,
             const std::vector<bool> &count, int flags, std::vector<cplx> &f,
             std::vector<TargetFunctionAtomicParamDerivatives> *dparam)
    {
        const size_t n = (size_t)n_atoms_;
        if (atoms.size() != n) throw Error("atom count differs from the calculator's");
        if (!count.empty() && count.size() != n) throw Error("countAtomContribution size differs from the atom count");
        if (!have_hkl_ || hkl != hkl_) setHkl(hkl);  // the set stays resident between calls
        atoms_ = atoms;
        std::vector<double> xyz(3 * n), adp(6 * n, 0.0), occ(n), dx(3 * n), dadp(6 * n), docc(n);
        std::vector<int> inc(n, 1);
        for (size_t a = 0; a < n; a++) {
            for (int k = 0; k < 3; k++) xyz[3 * a + k] = atoms[a].coordinates[k];
            if (atoms[a].adp.size() != (size_t)nadp_[a]) throw Error("ADP component count differs from the calculator's");
            for (size_t k = 0; k < atoms[a].adp.size(); k++) adp[6 * a + k] = atoms[a].adp[k];
            occ[a] = atoms[a].occupancy;
            if (!count.empty()) inc[a] = count[a] ? 1 : 0;
        }
        f.assign(hkl.size(), cplx(0.0, 0.0));
        dsf_outputs out{reinterpret_cast<double *>(f.data()), dx.data(), dadp.data(), docc.data(),
                        nullptr, nullptr, nullptr, nullptr};
        engine_->check(dsf_calculate_atoms(s_, precision_, flags, xyz.data(), adp.data(), occ.data(),
                                           reinterpret_cast<const double *>(dtdf.data()), inc.data(), &out),
                       "calculateStructureFactorsAndDerivatives");
        if (!dparam) return;
        dparam->resize(n);
        for (size_t a = 0; a < n; a++) {
            auto &d = (*dparam)[a];
            for (int k = 0; k < 3; k++) d.atomic_position_derivatives[k] = dx[3 * a + k];
            d.adp_derivatives.assign(dadp.begin() + 6 * a, dadp.begin() + 6 * a + nadp_[a]);
            d.occupancy_derivatives = docc[a];
        }
    }
};

// HansenCoppensStructureFactorCalculator (HansenCoppensStructureFactorCalculator.h:42-165)
class HcCalculator : public SfCalculator {
public:
    HcCalculator(std::shared_ptr<Engine> engine, const dsf_symmetry &sym, const dsf_hc_model &model,
                 const dsf_atoms &atoms)
        : SfCalculator(std::move(engine), atoms)
    {
        engine_->check(dsf_structure_create_hc(engine_->get(), &sym, &model, &atoms, &s_), "create_hc");
    }
    // setElectronScattering: wfn_z, wfn_f000 per wavefunction type (the electron scattering factor at s = 0)
    void setElectronScattering(bool on, const std::vector<int> &wfn_z = {}, const std::vector<double> &wfn_f000 = {})
    {
        engine_->check(dsf_structure_set_electron(s_, on ? 1 : 0, on ? wfn_z.data() : nullptr,
                                                  on ? wfn_f000.data() : nullptr),
                       "setElectronScattering");
    }
    // the point-group split of the deformation valence (EngineSymm) is always applied; nothing to switch
    void set_def_val_symm(bool) {}
    // AnyHcCalculator::getModelInformation (src/Scattering/AnyHcCalculator.cpp:28-34)
    void getModelInformation(std::vector<std::pair<std::string, std::string> > &modelInfo) const override
    {
        modelInfo.assign(1, {"SCATTERING MODEL", "Hansen-Coppens multipole model"});
    }
    std::string name() const override { return "hc_gb300"; }
};

// AnyIamCalculator (src/Scattering/AnyIamCalculator.cpp:49-154)
class IamCalculator : public SfCalculator {
public:
    // table: the name of the Gaussian parameterisation the caller filled dsf_iam_model from
    IamCalculator(std::shared_ptr<Engine> engine, const dsf_symmetry &sym, const dsf_iam_model &model,
                  const dsf_atoms &atoms, const std::string &table = std::string())
        : SfCalculator(std::move(engine), atoms), table_(table)
    {
        engine_->check(dsf_structure_create_iam(engine_->get(), &sym, &model, &atoms, &s_), "create_iam");
    }
    // AnyIamCalculator's model information (src/Scattering/AnyIamCalculator.cpp:55-56, 147)
    void getModelInformation(std::vector<std::pair<std::string, std::string> > &modelInfo) const override
    {
        modelInfo = {{"SCATTERING MODEL", "IAM"}, {"FORM FACTORS PARAMETERISATION", table_}};
    }
    std::string name() const override { return "iam_gb300"; }

private:
    std::string table_;
};

// TscFileBasedSfCalculator (src/Scattering/TscFileBasedSfCalculator.cpp:17-123): the reflection set of the
// structure is that of the file's expansion (h' = h R must be in the file for every h and operation)
class TscCalculator : public SfCalculator {
public:
    TscCalculator(std::shared_ptr<Engine> engine, const dsf_symmetry &sym, const dsf_atoms &atoms,
                  const std::vector<Vector3i> &hkl, const std::string &tsc_path)
        : SfCalculator(std::move(engine), atoms)
    {
        engine_->check(dsf_structure_create_tsc(engine_->get(), &sym, &atoms, (int)hkl.size(),
                                                hkl.empty() ? nullptr : hkl[0].data(), tsc_path.c_str(), &s_),
                       "create_tsc");
        hkl_ = hkl;
        have_hkl_ = true;
    }
    // TscFileBasedSfCalculator reports no model information (TscFileBasedSfCalculator.h:27)
    std::string name() const override { return "tsc_gb300"; }
};

}  // namespace dsf
