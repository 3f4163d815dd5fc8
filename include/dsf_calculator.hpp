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
 *   HcCalculator::setLocalCoordinateSystems(definitions, frozen, atoms): the LCS recomputed from the atoms
 *       on every update and calculation unless frozen     AnyHcCalculator.cpp:236-244, 319-329
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

#include <algorithm>
#include <array>
#include <cmath>
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

    // the atoms of the following single-h and form-factor calls (SfCalculator::update); an HC calculator with
    // local coordinate systems that are not frozen also recomputes them from these positions
    void update(const std::vector<AtomInCrystal> &atoms)
    {
        if (atoms.size() != (size_t)n_atoms_) throw Error("atom count differs from the calculator's");
        atoms_ = atoms;
        atomsChanged(atoms);
    }

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
    int atomCount() const { return n_atoms_; }
    const std::shared_ptr<Engine> &engine() const { return engine_; }
    const std::vector<int> &adpComponents() const { return nadp_; }
    int precision() const { return precision_; }
    // makes hkl the resident reflection set (no transfer when it already is)
    void setReflections(const std::vector<Vector3i> &hkl)
    {
        if (!have_hkl_ || hkl != hkl_) setHkl(hkl);
    }

protected:
    SfCalculator(std::shared_ptr<Engine> engine, const dsf_atoms &atoms) : engine_(std::move(engine)), n_atoms_(atoms.n_atoms)
    {
        nadp_.assign(atoms.adp_components, atoms.adp_components + atoms.n_atoms);
    }
    std::shared_ptr<Engine> engine_;
    dsf_structure *s_ = nullptr;
    std::vector<Vector3i> hkl_;
    bool have_hkl_ = false;

    // called with the atoms of every update and every calculation, before the engine sees them
    virtual void atomsChanged(const std::vector<AtomInCrystal> &) {}

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
        atomsChanged(atoms);
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

// fractional -> Cartesian matrix of a cell (a b c [A], alpha beta gamma [deg]): a along x, b in the xy plane, as
// the reference's UnitCell (src/CrystalStructure/UnitCell.cpp:183-212); row-major, r_cart = M r_frac
inline std::array<double, 9> fractionalToCartesian(const double cell[6])
{
    const double d = 3.14159265358979323846 / 180.0;
    const double ca = std::cos(cell[3] * d), cb = std::cos(cell[4] * d), cg = std::cos(cell[5] * d);
    const double sg = std::sin(cell[5] * d);
    const double v = std::sqrt(1.0 - ca * ca - cb * cb - cg * cg + 2.0 * ca * cb * cg);
    return {cell[0], cell[1] * cg, cell[2] * cb,
            0.0, cell[1] * sg, cell[2] * (ca - cb * cg) / sg,
            0.0, 0.0, cell[2] * v / sg};
}

// An XD-style local coordinate system of one atom, as the reference's XdLocalCoordinateSystem defines it
// (src/HC_Model/XdLocalCoordinateSystem.cpp:86-135, 220-288) with the axes of its CrossProductLcs
// (src/MathUtilities/CrossProductLcs.cpp:10-60): axis1 points from the central atom to point 1; axis2 lies in the
// plane of that direction and the auxiliary direction point2_to - point2_from, on its side; the third axis
// completes a right- (or left-) handed system.  A point given by several atoms is the SUM of their positions,
// as the reference computes it (averageAtomSetPosition adds the positions and does not divide); an empty list
// takes the fractional dummy position instead.
struct XdLcs {
    int central = -1;                              // atom index; -1: the Cartesian axes themselves
    std::vector<int> point1, point2_from, point2_to;
    Vector3d dummy1{}, dummy2_from{}, dummy2_to{};  // fractional, for empty point lists
    int axis1 = 3;                                  // +-1, +-2, +-3 for +-X, +-Y, +-Z
    int axis2 = 1;
    bool right_handed = true;
};

// the matrix of one system for the given atom positions (crystal's xyz convention; M from
// fractionalToCartesian): row-major, columns = local x, y, z in the Cartesian frame (the layout of dsf_atoms.lcs)
inline std::array<double, 9> lcsMatrix(const XdLcs &def, const std::array<double, 9> &M, bool cartesian_xyz,
                                       const std::vector<AtomInCrystal> &atoms)
{
    if (def.central < 0) return {1, 0, 0, 0, 1, 0, 0, 0, 1};
    auto mul = [&](const Vector3d &f) {
        return Vector3d{M[0] * f[0] + M[1] * f[1] + M[2] * f[2], M[3] * f[0] + M[4] * f[1] + M[5] * f[2],
                        M[6] * f[0] + M[7] * f[1] + M[8] * f[2]};
    };
    auto cart = [&](const Vector3d &x) { return cartesian_xyz ? x : mul(x); };
    auto point = [&](const std::vector<int> &list, const Vector3d &dummy) {
        if (list.empty()) return mul(dummy);
        Vector3d sum{0, 0, 0};
        for (int a : list) {
            if (a < 0 || a >= (int)atoms.size()) throw Error("local coordinate system refers to a missing atom");
            const Vector3d c = cart(atoms[a].coordinates);
            for (int k = 0; k < 3; k++) sum[k] += c[k];
        }
        return sum;
    };
    if (def.central >= (int)atoms.size()) throw Error("local coordinate system refers to a missing atom");
    const int c1 = std::abs(def.axis1), c2 = std::abs(def.axis2), c3 = 6 - c1 - c2;
    if (c1 < 1 || c1 > 3 || c2 < 1 || c2 > 3 || c1 == c2) throw Error("local coordinate system axes must differ");
    const Vector3d o = cart(atoms[def.central].coordinates), p1 = point(def.point1, def.dummy1);
    const Vector3d pa = point(def.point2_from, def.dummy2_from), pb = point(def.point2_to, def.dummy2_to);
    auto cross = [](const Vector3d &a, const Vector3d &b) {
        return Vector3d{a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    };
    auto unit = [](Vector3d v) {
        const double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (!(n > 0)) throw Error("degenerate local coordinate system");
        for (double &x : v) x /= n;
        return v;
    };
    const double s1 = def.axis1 > 0 ? 1.0 : -1.0, s2 = def.axis2 > 0 ? 1.0 : -1.0;
    // sign that keeps (axis1, axis2, axis3) right-handed for a cyclic or anticyclic order of the axis indices
    const double hand = (def.right_handed ? 1.0 : -1.0) * (1 - 2 * ((2 + c2 - c1) % 3));
    const Vector3d e1 = unit({s1 * (p1[0] - o[0]), s1 * (p1[1] - o[1]), s1 * (p1[2] - o[2])});
    const Vector3d aux{s2 * (pb[0] - pa[0]), s2 * (pb[1] - pa[1]), s2 * (pb[2] - pa[2])};
    Vector3d e3 = unit(cross(e1, aux));
    for (double &x : e3) x *= hand;
    Vector3d e2 = cross(e3, e1);
    for (double &x : e2) x *= hand;
    Vector3d axes[3];
    axes[c1 - 1] = e1;
    axes[c2 - 1] = e2;
    axes[c3 - 1] = e3;
    std::array<double, 9> m{};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) m[3 * i + j] = axes[j][i];
    return m;
}

// HansenCoppensStructureFactorCalculator (HansenCoppensStructureFactorCalculator.h:42-165); with local coordinate
// systems given as definitions, the LCS handling of AnyHcCalculator (src/Scattering/AnyHcCalculator.cpp:13-26,
// 218-244, 319-329)
class HcCalculator : public SfCalculator {
public:
    HcCalculator(std::shared_ptr<Engine> engine, const dsf_symmetry &sym, const dsf_hc_model &model,
                 const dsf_atoms &atoms)
        : SfCalculator(std::move(engine), atoms), M_(fractionalToCartesian(sym.cell)),
          cartesian_xyz_(atoms.xyz_convention == DSF_XYZ_CARTESIAN)
    {
        engine_->check(dsf_structure_create_hc(engine_->get(), &sym, &model, &atoms, &s_), "create_hc");
        if (atoms.lcs) lcs_.assign(atoms.lcs, atoms.lcs + 9 * (size_t)atoms.n_atoms);
    }
    // AnyHcCalculator's lcs and frozenLcs: unless frozen, every update(atoms) and every calculation with atoms
    // recomputes each atom's system from the positions it is given, and the engine gets the new matrices
    // (dsf_structure_set_lcs) when any of them changed; the calculation then uses them, as the reference's
    // update before its engine call does.  Frozen: the systems stay as they are (the reference computes them
    // once, at set-up; so does this call, from atoms).
    void setLocalCoordinateSystems(const std::vector<XdLcs> &lcs, bool frozen,
                                   const std::vector<AtomInCrystal> &atoms)
    {
        if (lcs.size() != atoms.size()) throw Error("one local coordinate system per atom is needed");
        lcs_defs_ = lcs;
        frozen_ = false;
        atomsChanged(atoms);
        frozen_ = frozen;
    }
    // the matrices the engine holds now ([n][3][3], columns = local x, y, z)
    const std::vector<double> &localCoordinateSystems() const { return lcs_; }
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

protected:
    void atomsChanged(const std::vector<AtomInCrystal> &atoms) override
    {
        if (lcs_defs_.empty() || frozen_) return;
        std::vector<double> m(9 * atoms.size());
        for (size_t a = 0; a < atoms.size(); a++) {
            const std::array<double, 9> q = lcsMatrix(lcs_defs_[a], M_, cartesian_xyz_, atoms);
            std::copy(q.begin(), q.end(), m.begin() + 9 * a);
        }
        if (m == lcs_) return;  // unchanged geometry: the engine keeps its P_lm
        engine_->check(dsf_structure_set_lcs(s_, m.data()), "set local coordinate systems");
        lcs_.swap(m);
    }

private:
    std::array<double, 9> M_;
    bool cartesian_xyz_;
    std::vector<XdLcs> lcs_defs_;
    bool frozen_ = false;
    std::vector<double> lcs_;
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

// CombinedStructureFactorCalculator (include/discamb/Scattering/CombinedStructureFactorCalculator.h:14-60,
// src/Scattering/CombinedStructureFactorCalculator.cpp): the atoms split over calculators (TAAM: the multipolar
// atoms on an HcCalculator, the others on an IamCalculator, HcAtomBankStructureFactorCalculator.cpp:482-499), F
// summed over them and every atom's derivatives taken from its own calculator.  Here each part is a calculator
// over its own atoms only (the reference masks the other atoms out of whole-crystal calculators), and the parts
// run in one batched submission (dsf_calculate_batch_atoms).  As the reference's set(), building it sets every
// atom's anomalous dispersion to zero; setAnomalous hands the parts new per-atom values.
class CombinedCalculator {
public:
    // parts[i] computes the atoms atoms[i] (whole-structure indices, in the part's own atom order); every atom
    // belongs to exactly one part; the parts share one engine
    CombinedCalculator(std::vector<std::shared_ptr<SfCalculator> > parts, std::vector<std::vector<int> > atoms)
        : parts_(std::move(parts)), atoms_(std::move(atoms))
    {
        if (parts_.empty()) throw Error("a combined calculator needs at least one calculator");
        if (parts_.size() != atoms_.size()) throw Error("one atom list per calculator is needed");
        for (const auto &l : atoms_) n_ += (int)l.size();
        std::vector<int> seen((size_t)n_, 0);
        for (size_t p = 0; p < parts_.size(); p++) {
            if ((int)atoms_[p].size() != parts_[p]->atomCount()) throw Error("atom list size differs from its calculator's");
            for (int a : atoms_[p]) {
                if (a < 0 || a >= n_ || seen[a]++) throw Error("every atom must belong to exactly one calculator");
            }
        }
        setAnomalous(std::vector<cplx>((size_t)n_, cplx(0.0, 0.0)));
    }

    void setPrecision(int precision) { precision_ = precision; }

    // per-atom f' + i f'' in the whole structure's atom order (CombinedStructureFactorCalculator::setAnomalous)
    void setAnomalous(const std::vector<cplx> &anomalous)
    {
        if ((int)anomalous.size() != n_) throw Error("anomalous dispersion size differs from the atom count");
        for (size_t p = 0; p < parts_.size(); p++) {
            std::vector<cplx> a(atoms_[p].size());
            for (size_t k = 0; k < a.size(); k++) a[k] = anomalous[atoms_[p][k]];
            parts_[p]->setAnomalous(a);
        }
    }

    void calculateStructureFactorsAndDerivatives(const std::vector<AtomInCrystal> &atoms,
                                                 const std::vector<Vector3i> &hkl, std::vector<cplx> &f,
                                                 std::vector<TargetFunctionAtomicParamDerivatives> &dTarget_dparam,
                                                 const std::vector<cplx> &dTarget_df,
                                                 const std::vector<bool> &countAtomContribution)
    {
        run(atoms, hkl, dTarget_df, countAtomContribution, DSF_D_XYZ | DSF_D_ADP | DSF_D_OCC, f, &dTarget_dparam);
    }
    void calculateStructureFactors(const std::vector<AtomInCrystal> &atoms, const std::vector<Vector3i> &hkl,
                                   std::vector<cplx> &f, const std::vector<bool> &countAtomContribution)
    {
        run(atoms, hkl, std::vector<cplx>(hkl.size(), cplx(1.0, 0.0)), countAtomContribution, 0, f, nullptr);
    }

private:
    std::vector<std::shared_ptr<SfCalculator> > parts_;
    std::vector<std::vector<int> > atoms_;
    int n_ = 0;
    int precision_ = DSF_FP64;

    void run(const std::vector<AtomInCrystal> &atoms, const std::vector<Vector3i> &hkl, const std::vector<cplx> &dtdf,
             const std::vector<bool> &count, int flags, std::vector<cplx> &f,
             std::vector<TargetFunctionAtomicParamDerivatives> *dparam)
    {
        if ((int)atoms.size() != n_) throw Error("atom count differs from the calculator's");
        if (!count.empty() && (int)count.size() != n_) throw Error("countAtomContribution size differs from the atom count");
        if (dtdf.size() != hkl.size()) throw Error("dTarget_df and hkl sizes differ");
        const size_t np = parts_.size(), m = hkl.size();
        std::vector<std::vector<double> > xyz(np), adp(np), occ(np), fp(np), dx(np), da(np), dox(np);
        std::vector<std::vector<int> > inc(np);
        std::vector<dsf_structure *> st(np);
        std::vector<const double *> px(np), pa(np), po(np), pg(np, reinterpret_cast<const double *>(dtdf.data()));
        std::vector<const int *> pi(np);
        std::vector<dsf_outputs> out(np);
        for (size_t p = 0; p < np; p++) {
            parts_[p]->setReflections(hkl);
            const auto &idx = atoms_[p];
            const auto &nadp = parts_[p]->adpComponents();
            const size_t k = idx.size();
            xyz[p].resize(3 * k);
            adp[p].assign(6 * k, 0.0);
            occ[p].resize(k);
            inc[p].assign(k, 1);
            for (size_t j = 0; j < k; j++) {
                const AtomInCrystal &a = atoms[idx[j]];
                for (int q = 0; q < 3; q++) xyz[p][3 * j + q] = a.coordinates[q];
                if (a.adp.size() != (size_t)nadp[j]) throw Error("ADP component count differs from the calculator's");
                for (size_t q = 0; q < a.adp.size(); q++) adp[p][6 * j + q] = a.adp[q];
                occ[p][j] = a.occupancy;
                if (!count.empty()) inc[p][j] = count[idx[j]] ? 1 : 0;
            }
            fp[p].assign(2 * m, 0.0);
            dx[p].assign(3 * k, 0.0);
            da[p].assign(6 * k, 0.0);
            dox[p].assign(k, 0.0);
            st[p] = parts_[p]->structure();
            px[p] = xyz[p].data();
            pa[p] = adp[p].data();
            po[p] = occ[p].data();
            pi[p] = inc[p].data();
            out[p] = dsf_outputs{fp[p].data(), dx[p].data(), da[p].data(), dox[p].data(), nullptr, nullptr, nullptr,
                                 nullptr};
        }
        const int rc = dsf_calculate_batch_atoms(st.data(), (int)np, precision_, flags, px.data(), pa.data(), po.data(),
                                                 pg.data(), pi.data(), out.data());
        parts_[0]->engine()->check(rc, "combined calculation");
        f.assign(m, cplx(0.0, 0.0));
        for (size_t p = 0; p < np; p++)
            for (size_t i = 0; i < m; i++) f[i] += cplx(fp[p][2 * i], fp[p][2 * i + 1]);
        if (!dparam) return;
        dparam->resize((size_t)n_);
        for (size_t p = 0; p < np; p++) {
            const auto &nadp = parts_[p]->adpComponents();
            for (size_t j = 0; j < atoms_[p].size(); j++) {
                auto &d = (*dparam)[atoms_[p][j]];
                for (int q = 0; q < 3; q++) d.atomic_position_derivatives[q] = dx[p][3 * j + q];
                d.adp_derivatives.assign(da[p].begin() + 6 * j, da[p].begin() + 6 * j + nadp[j]);
                d.occupancy_derivatives = dox[p][j];
            }
        }
    }
};

}  // namespace dsf
