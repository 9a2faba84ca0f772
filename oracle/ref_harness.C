// Driver for the reference DynELA numerical core (test infrastructure only, never shipped).
//
// It builds a model through the same Structure/Material/Boundary/Solver calls a .dyn deck makes
// (Samples/Taylor/Taylor_Axi_Parametric.dyn:40-125 shows that sequence), because the .dyn
// interpreter needs bison/flex, which this machine lacks.  Everything it computes is the
// reference's own code: Domain::computeInternalForces (finiteElement/Domain.C:130-738),
// ExplicitSolverCH (finiteElement/ExplicitSolverCH.C:115-567), Solver::computeTimeStep
// (finiteElement/Solver.C:220-267), ...
//
// Commands (file formats are defined in oracle/dnl_io.py):
//   ref_harness run    <model> <out>          full solve via Structure::solve(), final state
//   ref_harness steps  <model> <out> <K>      the ExplicitSolverCH loop step by step (its private
//                                             methods, same order as ExplicitSolverCH.C:179-274),
//                                             recording Fint and dt for the first K steps
//   ref_harness forces <model> <state> <out>  inject nodal + integration-point state, then one
//                                             computeInternalMatrices + computeInternalForces
//   ref_harness bench  <model> <out> <K>      K steps of the loop, wall time only
//   ref_harness tables <out>                  element tables of ElQua4nAx, ElHex8n3D, ElQua4n2D,
//                                             ElTet4n3D, ElTet10n3D
//
// Run it with OMP_NUM_THREADS=1 for golden data: strategy 0 of Domain::computeInternalForces sums
// element forces under `omp critical`, so with several threads the summation order (and the last
// bits of Fint) depends on scheduling.

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdarg>
#include <cmath>
#include <chrono>
#include <iostream>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>
#include <map>
#include <list>
#include <algorithm>
#include <omp.h>
#include <unistd.h>
#include <sys/types.h>
#include <sys/stat.h>

// The harness reads solver internals (increment counters, private steps of ExplicitSolverCH).
#define private public
#define protected public
#include <Structure.h>
#include <Domain.h>
#include <Node.h>
#include <NodalField.h>
#include <Element.h>
#include <ElQua4nAx.h>
#include <ElQua4n2D.h>
#include <ElTet4n3D.h>
#include <ElTet10n3D.h>
#include <ElHex8n3D.h>
#include <Material.h>
#include <IsoHardElastoplastic.h>
#include <Boundary.h>
#include <Select.h>
#include <Solver.h>
#include <ExplicitSolverCH.h>
#include <IntegrationPoint.h>
#include <io_Structure.h>
#include <IsoHardElastoplasticTabular.h>
#include <IsoHardMetafor.h>
#include <DiscreteFunction.h>
#undef private
#undef protected

// ------------------------------------------------------------------------------------ file IO
struct Reader
{
  FILE *f;
  explicit Reader(const char *path)
  {
    f = fopen(path, "rb");
    if (!f)
    {
      fprintf(stderr, "ref_harness: cannot open %s\n", path);
      exit(2);
    }
  }
  ~Reader() { fclose(f); }
  long i64()
  {
    long v;
    if (fread(&v, 8, 1, f) != 1)
      fail();
    return v;
  }
  double f64()
  {
    double v;
    if (fread(&v, 8, 1, f) != 1)
      fail();
    return v;
  }
  void f64s(double *p, size_t n)
  {
    if (n && fread(p, 8, n, f) != n)
      fail();
  }
  void fail()
  {
    fprintf(stderr, "ref_harness: truncated input\n");
    exit(2);
  }
};

// Output: a sequence of named float64 records: [i64 name_len][name][i64 count][count doubles].
struct Writer
{
  FILE *f;
  explicit Writer(const std::string &path)
  {
    f = fopen(path.c_str(), "wb");
    if (!f)
    {
      fprintf(stderr, "ref_harness: cannot write %s\n", path.c_str());
      exit(2);
    }
  }
  ~Writer() { fclose(f); }
  void rec(const std::string &name, const double *p, size_t n)
  {
    long len = (long)name.size(), cnt = (long)n;
    fwrite(&len, 8, 1, f);
    fwrite(name.data(), 1, name.size(), f);
    fwrite(&cnt, 8, 1, f);
    if (n)
      fwrite(p, 8, n, f);
  }
  void rec(const std::string &name, const std::vector<double> &v) { rec(name, v.data(), v.size()); }
  void scalar(const std::string &name, double v) { rec(name, &v, 1); }
};

struct BCGroup
{
  long kind; // 0 restrain (val = 0/1 mask), 1 imposed speed
  double val[3];
  std::vector<long> nodes;
};

struct MatLaw
{
  double E, nu, rho;
  long law; // 0 IsoHardElastoplastic, 1 none (elastic), 2 IsoHardElastoplasticTabular, 3 IsoHardMetafor
  double P[8];
  std::vector<double> tx, ty;
};

static long nenOf(long etype) { return etype == 1 ? 8 : (etype == 4 ? 10 : 4); }

struct Model
{
  long etype; // 0 ElQua4nAx, 1 ElHex8n3D, 2 ElQua4n2D, 3 ElTet4n3D, 4 ElTet10n3D, 9 per element
  long N, E, nen;
  std::vector<double> coords; // N*3
  std::vector<long> conn;     // the elements' nodes one after another, 0-based
  std::vector<long> etypes;   // per element (etype 9: a domain of several element types)
  std::vector<long> first;    // E+1 offsets into conn
  double mat[6];              // E, nu, rho, A, B, n
  double v0[3];               // initial speed of every node
  std::vector<BCGroup> bcs;
  double tend, rho_b, safety, freq, method, nsaves;
  // optional: several materials, element materials, per-node initial velocity
  std::vector<MatLaw> mats;
  std::vector<long> elemMat;
  std::vector<double> vel;
};

static const long EXT_MAGIC = 0x584c4e44; // "DNLX"

static const long MODEL_MAGIC = 0x4d4c4e44; // "DNLM"

static Model readModel(const char *path)
{
  Reader r(path);
  Model m;
  if (r.i64() != MODEL_MAGIC)
  {
    fprintf(stderr, "ref_harness: %s is not a model file\n", path);
    exit(2);
  }
  m.etype = r.i64();
  m.N = r.i64();
  m.E = r.i64();
  m.coords.resize(m.N * 3);
  r.f64s(m.coords.data(), m.coords.size());
  // etype 9: the type of each element follows (a domain of one family mixing element types,
  // Domain.C:1042-1060), then each element's nodes
  m.etypes.assign(m.E, m.etype);
  if (m.etype == 9)
    for (long e = 0; e < m.E; e++)
      m.etypes[e] = r.i64();
  m.first.assign(m.E + 1, 0);
  for (long e = 0; e < m.E; e++)
    m.first[e + 1] = m.first[e] + nenOf(m.etypes[e]);
  m.nen = m.etype == 9 ? 0 : nenOf(m.etype);
  m.conn.resize(m.first[m.E]);
  for (size_t i = 0; i < m.conn.size(); i++)
    m.conn[i] = r.i64();
  r.f64s(m.mat, 6);
  r.f64s(m.v0, 3);
  long nbc = r.i64();
  for (long b = 0; b < nbc; b++)
  {
    BCGroup g;
    g.kind = r.i64();
    r.f64s(g.val, 3);
    long cnt = r.i64();
    g.nodes.resize(cnt);
    for (long i = 0; i < cnt; i++)
      g.nodes[i] = r.i64();
    m.bcs.push_back(g);
  }
  m.tend = r.f64();
  m.rho_b = r.f64();
  m.safety = r.f64();
  m.freq = r.f64();
  m.method = r.f64();
  m.nsaves = r.f64();
  long magic;
  if (fread(&magic, 8, 1, r.f) == 1 && magic == EXT_MAGIC)
  {
    long nmat = r.i64();
    for (long i = 0; i < nmat; i++)
    {
      MatLaw ml;
      ml.E = r.f64();
      ml.nu = r.f64();
      ml.rho = r.f64();
      ml.law = r.i64();
      r.f64s(ml.P, 8);
      long np = r.i64();
      ml.tx.resize(np);
      ml.ty.resize(np);
      r.f64s(ml.tx.data(), np);
      r.f64s(ml.ty.data(), np);
      m.mats.push_back(ml);
    }
    if (r.i64())
    {
      m.elemMat.resize(m.E);
      for (long e = 0; e < m.E; e++)
        m.elemMat[e] = r.i64();
    }
    if (r.i64())
    {
      m.vel.resize(3 * m.N);
      r.f64s(m.vel.data(), 3 * m.N);
    }
  }
  return m;
}

// ------------------------------------------------------------------------------ model build
struct Built
{
  Structure *st;
  Domain *dom;
  ExplicitSolverCH *solver;
};

static Built build(const Model &m)
{
  Built b;
  Structure *st = new Structure; // registers itself as Global_Structure
  for (long n = 0; n < m.N; n++)
    st->createNode(n + 1, m.coords[3 * n], m.coords[3 * n + 1], m.coords[3 * n + 2]);

  // as a deck does: setDefaultElement, then createElement; again at each change of element type
  long protoType = -1;
  ElementSet *els = new ElementSet;
  for (long e = 0; e < m.E; e++)
  {
    const long et = m.etypes[e], nen = nenOf(et);
    if (et != protoType)
    {
      Element *proto = (et == 0   ? (Element *)new ElQua4nAx(0)
                        : et == 2 ? (Element *)new ElQua4n2D(0)
                        : et == 3 ? (Element *)new ElTet4n3D(0)
                        : et == 4 ? (Element *)new ElTet10n3D(0)
                                  : (Element *)new ElHex8n3D(0));
      st->setDefaultElement(proto);
      protoType = et;
    }
    const long *c = &m.conn[m.first[e]];
    if (nen == 4)
      st->createElement(e + 1, (int)c[0] + 1, (int)c[1] + 1, (int)c[2] + 1, (int)c[3] + 1);
    else if (nen == 8)
      st->createElement(e + 1, (int)c[0] + 1, (int)c[1] + 1, (int)c[2] + 1, (int)c[3] + 1,
                        (int)c[4] + 1, (int)c[5] + 1, (int)c[6] + 1, (int)c[7] + 1);
    else
      st->createElement(e + 1, (int)c[0] + 1, (int)c[1] + 1, (int)c[2] + 1, (int)c[3] + 1,
                        (int)c[4] + 1, (int)c[5] + 1, (int)c[6] + 1, (int)c[7] + 1,
                        (int)c[8] + 1, (int)c[9] + 1);
    els->add(e + 1);
  }

  if (m.mats.empty())
  {
    Material *mat = new Material;
    IsoHardElastoplastic *hard = new IsoHardElastoplastic;
    hard->setYieldStress(m.mat[3]);
    hard->setHardParameter(m.mat[4]);
    hard->setHardExponent(m.mat[5]);
    st->addMaterial(mat);
    mat->setYoung(m.mat[0]);
    mat->setPoisson(m.mat[1]);
    mat->setDensity(m.mat[2]);
    mat->setHardening(hard);
    st->attachMaterialToElements(mat, els);
  }
  else
  {
    // one Material per entry, its hardening as a deck builds it (Samples/Traction/Traction.dyn:
    // DiscreteFunction + IsoHardElastoplasticTabular::setFunction; a material without hardening),
    // attached to the ElementSet of its elements
    for (size_t i = 0; i < m.mats.size(); i++)
    {
      const MatLaw &ml = m.mats[i];
      Material *mat = new Material;
      st->addMaterial(mat);
      mat->setYoung(ml.E);
      mat->setPoisson(ml.nu);
      mat->setDensity(ml.rho);
      if (ml.law == 0)
      {
        IsoHardElastoplastic *hard = new IsoHardElastoplastic;
        hard->setYieldStress(ml.P[0]);
        hard->setHardParameter(ml.P[1]);
        hard->setHardExponent(ml.P[2]);
        mat->setHardening(hard);
      }
      else if (ml.law == 2)
      {
        DiscreteFunction *fn = new DiscreteFunction;
        for (size_t k = 0; k < ml.tx.size(); k++)
          fn->add(ml.tx[k], ml.ty[k]);
        IsoHardElastoplasticTabular *hard = new IsoHardElastoplasticTabular;
        hard->setFunction(fn);
        mat->setHardening(hard);
      }
      else if (ml.law == 3)
      {
        IsoHardMetafor *hard = new IsoHardMetafor;
        for (int k = 0; k < 8; k++)
          hard->getConstitutiveParameter(k) = ml.P[k];
        mat->setHardening(hard);
      }
      ElementSet *es = new ElementSet;
      for (long e = 0; e < m.E; e++)
        if ((m.elemMat.empty() ? 0 : m.elemMat[e]) == (long)i)
          es->add(e + 1);
      st->attachMaterialToElements(mat, es);
    }
  }

  if (m.vel.empty())
  {
    NodeSet *all = new NodeSet;
    for (long n = 0; n < m.N; n++)
      all->add(n + 1);
    BoundarySpeed *ini = new BoundarySpeed;
    ini->set(m.v0[0], m.v0[1], m.v0[2]);
    st->attachInitialBC(ini, all);
  }
  else
  {
    // one BoundarySpeed per node that moves (applyInitial_V0 on node sets)
    for (long n = 0; n < m.N; n++)
    {
      const double *v = &m.vel[3 * n];
      if (v[0] == 0. && v[1] == 0. && v[2] == 0.)
        continue;
      NodeSet *one = new NodeSet;
      one->add(n + 1);
      BoundarySpeed *ini = new BoundarySpeed;
      ini->set(v[0], v[1], v[2]);
      st->attachInitialBC(ini, one);
    }
  }

  for (size_t g = 0; g < m.bcs.size(); g++)
  {
    NodeSet *ns = new NodeSet;
    for (size_t i = 0; i < m.bcs[g].nodes.size(); i++)
      ns->add(m.bcs[g].nodes[i] + 1);
    Boundary *bnd;
    if (m.bcs[g].kind == 0)
    {
      BoundaryRestrain *r = new BoundaryRestrain;
      r->set(m.bcs[g].val[0], m.bcs[g].val[1], m.bcs[g].val[2]);
      bnd = r;
    }
    else
    {
      BoundarySpeed *s = new BoundarySpeed;
      s->set(m.bcs[g].val[0], m.bcs[g].val[1], m.bcs[g].val[2]);
      bnd = s;
    }
    st->attachConstantBC(bnd, ns);
  }

  ExplicitSolverCH *solver = new ExplicitSolverCH;
  solver->setTimes(0, m.tend);
  st->setSaveTimes(0, m.tend, m.tend / m.nsaves);
  st->addSolver(solver);
  solver->setTimeStepMethod(m.method == 0 ? "Courant" : "Pulse");
  if (m.rho_b != 0.8182)
    solver->setDissipation(m.rho_b);
  solver->setTimeStepSafetyFactor(m.safety);
  solver->setComputeTimeStepFrequency((Indice)m.freq);

  st->initSolve();
  // as DynELA_solve's main (Applications/DynELA_solve/main.C:100-101)
  st->resultFile->setMode(Write);
  st->resultFile->incrementalFile() = True;
  b.st = st;
  b.dom = st->domains(0);
  b.solver = solver;
  return b;
}

// ------------------------------------------------------------------------------ state dumps
static void dumpNodes(Writer &w, Domain *d, const char *prefix)
{
  long N = d->nodes.size();
  std::vector<double> x(3 * N), du(3 * N), v(3 * N), a(3 * N), disp(3 * N), mass(N);
  for (long n = 0; n < N; n++)
  {
    Node *p = d->nodes(n);
    for (int j = 0; j < 3; j++)
    {
      x[3 * n + j] = p->coords(j);
      du[3 * n + j] = p->Current->delta_disp(j);
      v[3 * n + j] = p->Current->mat_speed(j);
      a[3 * n + j] = p->Current->dmat_speed(j);
      disp[3 * n + j] = p->Current->disp(j);
    }
    mass[n] = p->mass;
  }
  std::string s(prefix);
  w.rec(s + "coords", x);
  w.rec(s + "du", du);
  w.rec(s + "v", v);
  w.rec(s + "a", a);
  w.rec(s + "disp", disp);
  w.rec(s + "mass", mass);
}

static void dumpIPs(Writer &w, Domain *d, const char *prefix)
{
  long E = d->elements.size();
  std::vector<double> S, Eps, EpsPlas, p, evp, Sig, dEps, R, detJ;
  for (long e = 0; e < E; e++)
  {
    Element *pel = d->elements(e);
    for (long pt = 0; pt < pel->getNumberOfIntegrationPoints(); pt++)
    {
      pel->getIntegrationPoint(pt);
      IntegrationPoint *ip = pel->ref;
      for (int k = 0; k < 9; k++)
      {
        S.push_back(ip->S(k / 3, k % 3));
        Eps.push_back(ip->Eps(k / 3, k % 3));
        EpsPlas.push_back(ip->EpsPlas(k / 3, k % 3));
        Sig.push_back(ip->Sig(k / 3, k % 3));
        dEps.push_back(ip->dEps(k / 3, k % 3));
        R.push_back(ip->R(k / 3, k % 3));
      }
      p.push_back(ip->p);
      evp.push_back(ip->evp);
      detJ.push_back(ip->detJ);
    }
  }
  std::string s(prefix);
  w.rec(s + "S", S);
  w.rec(s + "Eps", Eps);
  w.rec(s + "EpsPlas", EpsPlas);
  w.rec(s + "p", p);
  w.rec(s + "evp", evp);
  w.rec(s + "Sig", Sig);
  w.rec(s + "dEps", dEps);
  w.rec(s + "R", R);
  w.rec(s + "detJ", detJ);
}

static void dumpFint(Writer &w, Domain *d, const std::string &name)
{
  std::vector<double> f(d->Fint.size());
  for (long i = 0; i < (long)f.size(); i++)
    f[i] = d->Fint(i);
  w.rec(name, f);
}

// ------------------------------------------------------------------------------ commands
static int cmdRun(const Model &m, const std::string &out)
{
  Built b = build(m);
  auto t0 = std::chrono::steady_clock::now();
  b.st->solve();
  auto t1 = std::chrono::steady_clock::now();
  Writer w(out);
  dumpNodes(w, b.dom, "final_");
  dumpIPs(w, b.dom, "final_");
  w.scalar("time", b.dom->currentTime);
  w.scalar("increments", (double)b.solver->increment);
  w.scalar("wall_s", std::chrono::duration<double>(t1 - t0).count());
  w.scalar("threads", (double)omp_get_max_threads());
  return 0;
}

// The body of ExplicitSolverCH::solve (ExplicitSolverCH.C:115-278), same calls in the same order,
// with per-step records.  The history .plot line of endStep is written by the reference itself.
static int cmdSteps(const Model &m, const std::string &out, long K, bool record,
                    const char *resultsPath = nullptr)
{
  Built b = build(m);
  Domain *d = b.dom;
  ExplicitSolverCH *s = b.solver;
  Writer w(out);

  // Domain::solve prologue (Domain.C:1237-1288): history file, solver selection.
  d->history_file = fopen("dnlref.plot", "w");
  d->currentSolver = s;
  s->upTime = m.tend;
  if (!s->betweenTimeBounds())
    return 1;

  d->computeInternalMatrices();
  d->computeMassMatrix();
  d->computeInternalForces();
  s->computeTimeStep(True);
  if (record)
  {
    std::vector<double> mass(d->Mass.rows());
    for (long i = 0; i < (long)mass.size(); i++)
      mass[i] = d->Mass(i);
    w.rec("mass", mass);
    w.scalar("dt0", s->timeStep);
  }

  std::vector<double> dts, times, kin;
  double wall = 0;
  long k = 0;
  bool run = true;
  while (run && k < K)
  {
    auto t0 = std::chrono::steady_clock::now();
    s->initStep();
    s->computePredictions();
    s->initIteration();
    if (record)
    {
      char nm[64];
      sprintf(nm, "fint_%06ld", k);
      dumpFint(w, d, nm);
      dts.push_back(s->timeStep);
    }
    s->explicitSolve();
    // kinetic energy of the New field, as endStep writes it to the .plot file (ExplicitSolverCH.C:459-461)
    double ke = record ? d->getTotalKineticEnergy() : 0.0;
    s->endStep();
    if (!s->betweenTimeBounds())
      run = false;
    if (run)
    {
      d->computeInternalMatrices();
      s->computeTimeStep();
    }
    auto t1 = std::chrono::steady_clock::now();
    wall += std::chrono::duration<double>(t1 - t0).count();
    if (record)
    {
      times.push_back(d->currentTime);
      kin.push_back(ke);
    }
    k++;
  }
  if (record)
  {
    w.rec("dt", dts);
    w.rec("time", times);
    w.rec("kinetic", kin);
    dumpNodes(w, d, "final_");
    dumpIPs(w, d, "final_");
  }
  if (resultsPath)
  {
    // the reference's own binary results file (io_Data::structure_write, io_Data.C:486-506)
    // Structure::solve sets the structure's time to the domain's before each save (Structure.C:852)
    b.st->currentTime = d->currentTime;
    std::ofstream pf(resultsPath);
    b.st->writeData(pf);
  }
  w.scalar("steps", (double)k);
  w.scalar("wall_s", wall);
  w.scalar("threads", (double)omp_get_max_threads());
  w.scalar("elements", (double)d->elements.size());
  return 0;
}

// State file: per node coords(3) du(3) v(3) a(3) disp(3); per element, per IP: S(9) Eps(9)
// EpsPlas(9) p evp; then the solver timeStep.
static int cmdForces(const Model &m, const char *statePath, const std::string &out)
{
  Built b = build(m);
  Domain *d = b.dom;
  Reader r(statePath);
  if (r.i64() != 0x54534e44) // "DNST"
  {
    fprintf(stderr, "ref_harness: %s is not a state file\n", statePath);
    return 2;
  }
  for (long n = 0; n < d->nodes.size(); n++)
  {
    Node *p = d->nodes(n);
    double buf[15];
    r.f64s(buf, 15);
    for (int j = 0; j < 3; j++)
    {
      p->coords(j) = buf[j];
      p->Current->delta_disp(j) = buf[3 + j];
      p->Current->mat_speed(j) = buf[6 + j];
      p->Current->dmat_speed(j) = buf[9 + j];
      p->Current->disp(j) = buf[12 + j];
    }
  }
  for (long e = 0; e < d->elements.size(); e++)
  {
    Element *pel = d->elements(e);
    for (long pt = 0; pt < pel->getNumberOfIntegrationPoints(); pt++)
    {
      pel->getIntegrationPoint(pt);
      IntegrationPoint *ip = pel->ref;
      double buf[29];
      r.f64s(buf, 29);
      for (int k = 0; k < 9; k++)
      {
        ip->S(k / 3, k % 3) = buf[k];
        ip->Eps(k / 3, k % 3) = buf[9 + k];
        ip->EpsPlas(k / 3, k % 3) = buf[18 + k];
      }
      ip->p = buf[27];
      ip->evp = buf[28];
    }
  }
  d->currentSolver = b.solver;
  b.solver->timeStep = r.f64();
  d->computeInternalMatrices();
  d->computeInternalForces();
  Writer w(out);
  dumpFint(w, d, "fint");
  dumpIPs(w, d, "out_");
  return 0;
}

// Element tables of ElQua4nAx / ElHex8n3D / ElQua4n2D / ElTet4n3D / ElTet10n3D (ElQua4nAx.C:31-101,
// ElHex8n3D.C:26-161, ElQua4n2D.C:26-70, ElTet4n3D.C:33-57, ElTet10n3D.C:31-77): per Gauss point
// its weight, N_k and dN_k/dxi_c, as the compiled tables hold them.
static int cmdTables(const std::string &out)
{
  Writer w(out);
  const ElementData *tabs[5] = {&ElQua4nAx::elementData, &ElHex8n3D::elementData,
                                &ElQua4n2D::elementData, &ElTet4n3D::elementData,
                                &ElTet10n3D::elementData};
  const char *names[5] = {"axi", "hex", "plane", "tet4", "tet10"};
  for (int t = 0; t < 5; t++)
  {
    const ElementData *d = tabs[t];
    std::vector<double> wgt, N, dN;
    for (int pt = 0; pt < d->numberOfIntegrationPoints; pt++)
    {
      const ElementIntegrationPoint &ip = d->integrationPoint[pt];
      wgt.push_back(ip.weight);
      for (int k = 0; k < d->numberOfNodes; k++)
      {
        N.push_back(ip.shapeFunction(k));
        for (int c = 0; c < d->numberOfDimensions; c++)
          dN.push_back(ip.derShapeFunction(k, c));
      }
    }
    w.rec(std::string(names[t]) + "_weight", wgt);
    w.rec(std::string(names[t]) + "_N", N);
    w.rec(std::string(names[t]) + "_dN", dN);
  }
  return 0;
}

int main(int argc, char **argv)
{
  if (argc == 3 && std::string(argv[1]) == "tables")
    return cmdTables(argv[2]);
  if (argc < 4)
  {
    fprintf(stderr, "usage: ref_harness run|steps|forces|bench <model> ...\n");
    return 2;
  }
  std::string cmd = argv[1];
  Model m = readModel(argv[2]);
  if (cmd == "run")
    return cmdRun(m, argv[3]);
  if (cmd == "steps" && argc >= 6)
    return cmdSteps(m, argv[3], atol(argv[4]), true, argv[5]);
  if (cmd == "steps" && argc >= 5)
    return cmdSteps(m, argv[3], atol(argv[4]), true);
  if (cmd == "bench" && argc >= 5)
    return cmdSteps(m, argv[3], atol(argv[4]), false);
  if (cmd == "forces" && argc >= 5)
    return cmdForces(m, argv[3], argv[4]);
  fprintf(stderr, "ref_harness: bad command\n");
  return 2;
}
