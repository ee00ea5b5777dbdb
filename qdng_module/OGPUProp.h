// OGPUProp.h -- QDng propagator modules running on the GB300 engine.
//
// A QDng operator module (libqd-O<Name>.so, loaded by QDng's ModuleLoader,
// src/modules/ModuleLoader.h:193-243) that replaces one of OCheby, OGSPO,
// OSIL or OArnoldi.  Init(WaveFunction*) walks the Hamiltonian the way the
// reference propagators find it -- the child "hamiltonian" for Cheby, SIL
// and Arnoldi, the members "A", "B", ... for GSPO (src/qdlib/OGSPO.cpp:61-104)
// -- and hands the grid operators to the engine through its C ABI
// (include/qdg.h).  Apply(WaveFunction*) is one time step on the device with
// the host wave function authoritative: copied in, stepped, copied back.
// Operators the engine does not cover raise EIncompatible: there is no CPU
// fallback.  Engine status codes become QDng exceptions (EParamProblem,
// EIncompatible, EOverflow, EIOError; src/tools/Exception.h).
//
// Built against the QDng headers (same compiler ABI) and linked with
// libqdg.so; one .cpp per propagator name (OGPUCheby.cpp, OGPUGSPO.cpp,
// OGPUSIL.cpp, OGPUArnoldi.cpp).  XML: the reference's <propagator> node with
// name="GPUCheby" etc. and the same attributes, plus an optional
// precision="fp64|df64|mixed" (default fp64, binary64 throughout).
#ifndef QDNG_GB300_OGPUPROP_H
#define QDNG_GB300_OGPUPROP_H

#include <sstream>
#include <string>
#include <vector>

#include "modules/Module.h"
#include "qdg.h"
#include "qdlib/ODSpace.h"
#include "qdlib/OGobbler.h"
#include "qdlib/OGridDipole.h"
#include "qdlib/OGridGMat.h"
#include "qdlib/OGridHOFD.h"
#include "qdlib/OGridNAC.h"
#include "qdlib/OGridNablaSq.h"
#include "qdlib/OGridPotential.h"
#include "qdlib/OMultistate.h"
#include "qdlib/OPropagator.h"
#include "qdlib/OSum.h"
#include "qdlib/WFGridSystem.h"
#include "qdlib/WFMultistate.h"
#include "tools/Exception.h"

namespace QDLIB {

class OGPUProp : public OPropagator {
 protected:
  string _name;
  const char *_method;  // engine propagator: "Cheby", "GSPO", "SIL" or "Arnoldi"
  qdg_plan *_plan = nullptr;
  qdg_prop *_prop = nullptr;
  qdg_wf *_scratch = nullptr;
  std::vector<qdg_hterm> _terms;
  std::vector<double> _grids, _lasers;
  int _laser_nt = 0;
  int _nstates = 1;
  bool _nonherm = false;
  WaveFunction *_proto = nullptr;  // grid of the plan (coupling grids are loaded onto it)

  static void check(qdg_status s) {
    if (s == QDG_OK) return;
    const char *m = qdg_last_error();
    if (s == QDG_EINVAL) throw EParamProblem(m);
    if (s == QDG_EUNSUPPORTED) throw EIncompatible(m);
    if (s == QDG_ENONFINITE) throw EOverflow(m);
    throw EIOError(m);
  }

  int add_grid(const dVec &v) {
    _grids.insert(_grids.end(), v.begin(0), v.begin(0) + v.size());
    return int(_grids.size() / v.size()) - 1;
  }

  int add_laser(Laser *l) {
    if (_laser_nt == 0) _laser_nt = l->size();
    if (l->size() != _laser_nt) throw EIncompatible("GPU propagator: laser fields of different length");
    _lasers.insert(_lasers.end(), l->begin(0), l->begin(0) + l->size());
    return int(_lasers.size() / _laser_nt) - 1;
  }

  // One element H_{row,col} (or a GSPO member's element): a Sum or one grid operator.
  void collect(Operator *O, int row, int col, int group) {
    if (OSum *s = dynamic_cast<OSum *>(O)) {
      for (int i = 0; i < s->Size(); i++) collect(s->Get(i), row, col, group);
      return;
    }
    qdg_hterm t = {};
    t.row = row;
    t.col = col;
    t.grid = -1;
    t.laser = -1;
    t.group = group;
    if (OGridNAC *N = dynamic_cast<OGridNAC *>(O)) {
      // OGridNAC keeps its coupling grids private; load them the way its
      // Init(ParamContainer&) does (OGridNAC.cpp:30-87): file<d> per
      // dimension (the file itself for a 1-D NAC with a mass), sign, mass
      ParamContainer &np = N->Params();
      string file;
      np.GetValue("file", file);
      int dims = 1;
      if (np.isPresent("dims")) np.GetValue("dims", dims);
      t.kind = QDG_TERM_NAC;
      t.mass[0] = 1;
      t.sign = 1;
      if (np.isPresent("sign")) np.GetValue("sign", t.sign);
      const bool mass1d = dims == 1 && np.isPresent("mass");
      if (mass1d) np.GetValue("mass", t.mass[0]);
      for (int d = 0; d < dims; d++) {
        ParamContainer pf;
        std::ostringstream fn;
        fn << file;
        if (!mass1d) fn << d;
        pf.SetValue("file", fn.str());
        OGridPotential f;
        f.Init(pf);
        f.Init(_proto);
        const int g = add_grid(static_cast<dVec &>(f));
        if (d == 0) t.grid = g;
      }
    } else if (OGridNablaSq *T = dynamic_cast<OGridNablaSq *>(O)) {
      ParamContainer &tp = T->Params();
      vector<double> m;
      tp.GetArray("mass", m);
      t.kind = QDG_TERM_KINETIC;
      for (size_t d = 0; d < m.size() && d < QDG_MAX_DIMS; d++) t.mass[d] = m[d];
      // method, order and pbc as Diff::InitParams reads them (Diff.cpp:149-200)
      string method = "FFT";
      if (tp.isPresent("method")) tp.GetValue("method", method);
      if (method == "HOFD") {
        int order = 8;  // DIFF_DEF_ORDER (Diff.h:20)
        if (tp.isPresent("order")) tp.GetValue("order", order);
        bool pbc;
        tp.GetValue("pbc", pbc, false);
        t.fd_order = order;
        t.flags = pbc ? 1 : 0;
      } else if (method != "FFT") {
        throw EParamProblem("Unknown differenciation method", method);
      }
    } else if (OGobbler *Gb = dynamic_cast<OGobbler *>(O)) {
      // the filter grid W, gain included, is built by OGobbler::Init(WaveFunction*)
      // (OGobbler.cpp:118-185); nip and gain as OGobbler::Init(ParamContainer&) reads them
      Gb->Init(_proto);
      ParamContainer &bp = Gb->Params();
      bool nip;
      bp.GetValue("nip", nip, false);
      double gain = 1;
      if (bp.isPresent("gain")) bp.GetValue("gain", gain);
      t.kind = QDG_TERM_GOBBLER;
      t.grid = add_grid(static_cast<dVec &>(*Gb));
      t.laser = nip ? 1 : 0;
      t.mass[0] = gain;
    } else if (OGridHOFD *Hf = dynamic_cast<OGridHOFD *>(O)) {
      // deriv, order, dim, pbc and mass as OGridHOFD::Init reads them
      // (OGridHOFD.cpp:32-95; defaults deriv 1, order 2, all dimensions)
      ParamContainer &hp = Hf->Params();
      int deriv = 1, order = 2, dim = -1;
      bool pbc;
      if (hp.isPresent("deriv")) hp.GetValue("deriv", deriv);
      if (hp.isPresent("order")) hp.GetValue("order", order);
      if (hp.isPresent("dim")) hp.GetValue("dim", dim);
      hp.GetValue("pbc", pbc, false);
      t.kind = QDG_TERM_HOFD;
      t.fd_order = order;
      t.laser = dim;
      t.flags = (pbc ? 1 : 0) | (deriv == 1 ? 2 : 0);
      if (deriv != 1 && deriv != 2) throw EParamProblem("Invalid FD derivative", deriv);
      if (hp.isPresent("mass")) {
        vector<double> m;
        hp.GetArray("mass", m);
        t.flags |= 4;
        for (size_t d = 0; d < m.size() && d < QDG_MAX_DIMS; d++) t.mass[d] = m[d];
      }
    } else if (OGridGMat *Gm = dynamic_cast<OGridGMat *>(O)) {
      // OGridGMat keeps its elements private: read them the way its
      // Init(ParamContainer&) does (OGridGMat.cpp:142-248), lower triangle row by row
      ParamContainer &gp = Gm->Params();
      int n = 0;
      gp.GetValue("dims", n);
      bool coup, chain, pml;
      gp.GetValue("coup", coup, true);
      gp.GetValue("chainrule", chain, false);
      gp.GetValue("pml", pml, false);
      string method = "FFT";
      if (gp.isPresent("method")) gp.GetValue("method", method);
      if (chain || pml || method != "FFT")
        throw EIncompatible("GPU propagator: GridGMat with chain rule, PML or finite differences", O->Name());
      const int ne = n * (n + 1) / 2;
      vector<char> src(ne, gp.isPresent("G") ? 'c' : 'g');
      if (gp.isPresent("Gdef")) {
        vector<char> v;
        gp.GetArray("Gdef", v);
        for (size_t k = 0; k < v.size() && (int)k < ne; k++) src[k] = v[k];
      }
      vector<double> gc(ne, 0.0);
      if (gp.isPresent("G")) {
        vector<double> v;
        gp.GetArray("G", v);
        for (size_t k = 0; k < v.size() && (int)k < ne; k++) gc[k] = v[k];
      }
      string name;
      gp.GetValue("gmat", name);
      t.kind = QDG_TERM_GMAT;
      for (int i = 0, k = 0; i < n; i++)
        for (int j = 0; j <= i; j++, k++) {
          int code = (i != j && !coup) ? 0 : src[k] == 'g' ? 1 : src[k] == 'c' ? 2 : 0;
          dVec vals(_proto->size());
          vals = code == 2 ? gc[k] : 0.0;
          int g;
          if (code == 1) {
            if (name.length() < 2) throw EParamProblem("No G-matrix elements given");
            std::ostringstream fn;
            fn << name << "_" << i << j;
            ParamContainer pf;
            pf.SetValue("file", fn.str());
            OGridPotential f;
            f.Init(pf);
            f.Init(_proto);
            g = add_grid(static_cast<dVec &>(f));
          } else {
            g = add_grid(vals);
          }
          if (k == 0) t.grid = g;
          t.flags |= code << (2 * k);
        }
    } else if (OGridDipole *D = dynamic_cast<OGridDipole *>(O)) {  // before OGridPotential (its base)
      t.kind = QDG_TERM_DIPOLE;
      t.grid = add_grid(static_cast<dVec &>(*D));
      t.laser = add_laser(D->GetLaser());
    } else if (OGridPotential *V = dynamic_cast<OGridPotential *>(O)) {
      t.kind = QDG_TERM_POTENTIAL;
      t.grid = add_grid(static_cast<dVec &>(*V));
    } else {
      throw EIncompatible("GPU propagator: operator not on the GPU path", O->Name());
    }
    _terms.push_back(t);
  }

  // A Multistate matrix (every element as given; the engine applies QDng's
  // hermitian copy unless "nonhermitian" is set or both (i,j) and (j,i)
  // are given, OMultistate.cpp:52-53,83-85) or a single-state operator.
  void collect_tree(Operator *O, int group) {
    if (OMultistate *M = dynamic_cast<OMultistate *>(O)) {
      if (group > 0 && M->States() != _nstates) throw EIncompatible("GPU propagator: members of different state count");
      _nstates = M->States();
      bool nh = false;
      if (M->Params().isPresent("nonhermitian")) M->Params().GetValue("nonhermitian", nh);
      _nonherm = _nonherm || nh;
      for (int i = 0; i < M->States(); i++)
        for (int j = 0; j < M->States(); j++) {
          Operator *e = M->State(i, j);
          if (!e) continue;
          if (i > j && M->State(j, i) == e) continue;  // the hermitian pointer copy of (j, i)
          collect(e, i, j, group);
        }
    } else {
      collect(O, 0, 0, group);
    }
  }

  // The <propagator> attributes the reference propagator reads
  // (OCheby.cpp:53-61,386-401; OSIL.cpp:38-52; OArnoldi.cpp:39-59).
  std::string engine_params() {
    static const char *cheby[] = {"order", "prec", "scaling", "Emax", "Emax_im", "Emin", "Emin_im", nullptr};
    static const char *sil[] = {"order", "err", nullptr};
    static const char *arnoldi[] = {"order", "conv", nullptr};
    static const char *none[] = {nullptr};
    const string m(_method);
    const char **keys = m == "Cheby" ? cheby : m == "SIL" ? sil : m == "Arnoldi" ? arnoldi : none;
    std::ostringstream p;
    for (int i = 0; keys[i]; i++)
      if (_params.isPresent(keys[i])) {
        string v;
        _params.GetValue(keys[i], v);
        p << keys[i] << "=" << v << ";";
      }
    return p.str();
  }

  int engine_precision() {
    if (!_params.isPresent("precision")) return QDG_PREC_FP64;
    string v;
    _params.GetValue("precision", v);
    if (v == "fp64") return QDG_PREC_FP64;
    if (v == "df64") return QDG_PREC_DF64;
    if (v == "mixed") return QDG_PREC_MIXED;
    throw EParamProblem("GPU propagator: precision must be fp64, df64 or mixed");
  }

 public:
  OGPUProp(const char *name, const char *method) : _name(name), _method(method) {}
  ~OGPUProp() {
    qdg_wf_destroy(_scratch);
    qdg_prop_destroy(_prop);
    qdg_plan_destroy(_plan);
  }

  virtual const string &Name() { return _name; }
  virtual void Init(ParamContainer &params) { _params = params; }

  virtual void Init(WaveFunction *Psi) {
    OPropagator::Init(Psi);  // clock and dt checks (OPropagator.h:171-183)
    if (_plan) return;       // avoid init twice
    WFGridSystem *g = dynamic_cast<WFGridSystem *>(Psi);
    if (WFMultistate *ms = dynamic_cast<WFMultistate *>(Psi)) g = dynamic_cast<WFGridSystem *>(ms->State(0));
    if (!g) throw EIncompatible("GPU propagator needs a grid wave function");
    _proto = g;
    qdg_hplan_desc d = {};
    d.grid.ndims = g->Dim();
    for (int i = 0; i < g->Dim(); i++) {
      d.grid.n[i] = g->DimSize(i);
      d.grid.xmin[i] = g->Xmin(i);
      d.grid.xmax[i] = g->Xmax(i);
    }
    if (string(_method) == "GSPO") {
      // the split members A, B, C, ... (OGSPO.cpp:71-85); H is their sum
      H = new OSum();
      for (int i = 0; i < OList::Size(); i++) {
        char base[2] = "A";
        base[0] += i;
        Operator *O = Get(string(base));
        if (dynamic_cast<ODSpace *>(O) == nullptr)
          throw EIncompatible("GSPO: Operator has no diagonal representation", O->Name());
        collect_tree(O, i);
        dynamic_cast<OSum *>(H)->Add(string(base), O);
      }
    } else {
      H = Get("hamiltonian");
      collect_tree(H, 0);
    }
    d.nstates = _nstates;
    d.nonhermitian = _nonherm ? 1 : 0;
    d.nterms = (int32_t)_terms.size();
    d.terms = _terms.data();
    d.ngrids = _grids.empty() ? 0 : (int32_t)(_grids.size() / g->size());
    d.grid_data = _grids.data();
    d.nlasers = _laser_nt ? (int32_t)(_lasers.size() / _laser_nt) : 0;
    d.laser_nt = _laser_nt;
    d.laser_data = _lasers.data();
    check(qdg_plan_create(&d, engine_precision(), &_plan));
    const bool imag = Exponent().imag() == 0;
    const bool backward = imag ? Exponent().real() < 0 : Exponent().imag() > 0;
    check(qdg_prop_create(_plan, _method, engine_params().c_str(), clock->Dt(), imag, backward, &_prop));
    check(qdg_prop_init(_prop));
    check(qdg_wf_create(_plan, &_scratch));
  }

  // One step with psi authoritative on the host: each state's block is
  // copied to the device, stepped and copied back (QDng keeps one block per
  // state, WFMultistate.cpp:89-140).
  virtual void Apply(WaveFunction *Psi) {
    std::vector<double *> states;
    if (WFMultistate *ms = dynamic_cast<WFMultistate *>(Psi)) {
      for (int s = 0; s < ms->States(); s++) states.push_back((double *)ms->State(s)->begin(0));
    } else {
      states.push_back((double *)Psi->begin(0));
    }
    if ((int)states.size() != _nstates) throw EIncompatible("GPU propagator: wave function has the wrong state count");
    int32_t terms = 0;
    check(qdg_prop_apply_host_states(_prop, _scratch, states.data(), clock->TimeStep(), &terms));
  }

  virtual void Apply(WaveFunction *dest, WaveFunction *src) {
    *dest = src;
    Apply(dest);
  }
  virtual Operator *operator=(Operator *O) { return Copy(O); }
  virtual Operator *Copy(Operator *O) {
    OPropagator::Copy(O);
    return this;
  }
  virtual bool Valid(WaveFunction *Psi) { return H != nullptr && H->Valid(Psi); }
};

}  // namespace QDLIB

#endif
