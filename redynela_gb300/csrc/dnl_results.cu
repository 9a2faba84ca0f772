// Results / restart files in the reference's binary format.
//
// Layout (a stream of doubles, native byte order), as Structure::writeData (Structure.C:936-952)
// writes it through io_Data::structure_write (io_Data.C:486-506):
//   header      version (VERSION, RELEASE, UNDER_RELEASE) = (3, 1, 0), check (1.02, 0, 0)
//               (Structure::checkBinaryVersionWrite, Structure.C:990-1011; Const.h:43-46,
//               Structure.h:34)
//   time        Structure::currentTime (set to the domain's time before a save, Structure.C:852)
//   per domain  Domain::writeData (Domain.C:1407-1431):
//     header, time (Domain::currentTime)
//     per node  Node::write (Node.C:156-162): coords(3), then the Current NodalField
//               (NodalField.C:102-117): ro, dro, e, de, T, mat_speed(3), dmat_speed(3), fe(3),
//               delta_disp(3), disp(3)
//     separator (69, 0, 0) (Structure.h:35)
//     per element, per integration point: IntegrationPoint::write (IntegrationPoint.C:155-167):
//               p, evp, S(9), Sig(9), Eps(9), dEps(9), EpsPlas(9), tensors row-major
//     separator
//   separator (after each domain)
// The explicit path carries no thermal fields (dro, e, de, T are 0) and does not store nodal fe
// (0).  NodalField::ro holds the density on the field that was Current at Domain::initSolve only
// (Domain.C:1088) and the fields swap each step (Node.C:219-229), so the Current ro written is the
// density after an even number of steps and 0 after an odd number; the writer reproduces that.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "dnl_common.cuh"

namespace {

constexpr double kVersion[3] = {3., 1., 0.};
constexpr double kCheck = 1.02, kSeparator = 69.;

struct Out {
  FILE *f;
  bool ok = true;
  void put(const double *v, size_t n) { ok = ok && fwrite(v, sizeof(double), n, f) == n; }
  void put(double v) { put(&v, 1); }
  void header()
  {
    const double c[3] = {kCheck, 0., 0.};
    put(kVersion, 3);
    put(c, 3);
  }
  void separator()
  {
    const double c[3] = {kSeparator, 0., 0.};
    put(c, 3);
  }
};

struct In {
  const std::vector<double> &d;
  size_t at = 0;
  bool ok = true;
  explicit In(const std::vector<double> &data) : d(data) {}
  double get()
  {
    if (at >= d.size()) {
      ok = false;
      return 0.;
    }
    return d[at++];
  }
  void get(double *v, size_t n)
  {
    for (size_t i = 0; i < n; i++) v[i] = get();
  }
  void header()
  {
    double v[6];
    get(v, 6);
    ok = ok && v[0] == kVersion[0] && v[1] == kVersion[1] && v[2] == kVersion[2] && v[3] == kCheck;
  }
  void separator()
  {
    double v[3];
    get(v, 3);
    ok = ok && v[0] == kSeparator;
  }
};

}  // namespace

extern "C" {

int dnl_write_results(dnl_handle *h, const char *path)
{
  if (!h || !path || !h->stepT) return DNL_ERR_ARG;
  const long N = h->N, nIP = dnl::ip_total(h);  // every group's points, in element order
  std::vector<double> x(3 * N), du(3 * N), v(3 * N), a(3 * N), disp(3 * N);
  std::vector<double> S(9 * nIP), Eps(9 * nIP), EpsPlas(9 * nIP), p(nIP), evp(nIP), dE(9 * nIP);
  dnl_state_view sv;
  memset(&sv, 0, sizeof sv);
  sv.coords = x.data();
  sv.du = du.data();
  sv.v = v.data();
  sv.a = a.data();
  sv.disp = disp.data();
  sv.S = S.data();
  sv.Eps = Eps.data();
  sv.EpsPlas = EpsPlas.data();
  sv.p = p.data();
  sv.evp = evp.data();
  int r = dnl_get_state(h, &sv);
  if (r) return r;
  std::vector<double> R(9 * nIP);
  if ((r = dnl_get_step_tensors(h, dE.data(), R.data()))) return r;
  dnl_time_info t;
  if ((r = dnl_get_time_info(h, &t))) return r;
  FILE *f = fopen(path, "wb");
  if (!f) return DNL_ERR_ARG;
  Out o{f};
  o.header();
  o.put(t.time);
  o.header();
  o.put(t.time);
  for (long n = 0; n < N; n++) {
    o.put(&x[3 * n], 3);
    const double ro = h->cur != 0 ? 0. : (h->nodeRo ? h->nodeRo[n] : h->mat.rho);
    const double therm[5] = {ro, 0., 0., 0., 0.};  // ro, dro, e, de, T
    o.put(therm, 5);
    o.put(&v[3 * n], 3);
    o.put(&a[3 * n], 3);
    const double fe[3] = {0., 0., 0.};
    o.put(fe, 3);
    o.put(&du[3 * n], 3);
    o.put(&disp[3 * n], 3);
  }
  o.separator();
  const double I[9] = {1., 0., 0., 0., 1., 0., 0., 0., 1.};
  for (long q = 0; q < nIP; q++) {
    o.put(p[q]);
    o.put(evp[q]);
    double sig[9];
    for (int k = 0; k < 9; k++) sig[k] = S[9 * q + k] + p[q] * I[k];  // Sig = S + p I
    o.put(&S[9 * q], 9);
    o.put(sig, 9);
    o.put(&Eps[9 * q], 9);
    o.put(&dE[9 * q], 9);
    o.put(&EpsPlas[9 * q], 9);
  }
  o.separator();
  o.separator();
  const bool ok = o.ok;
  if (fclose(f) != 0 || !ok) return DNL_ERR_ARG;
  return 0;
}

int dnl_read_results(dnl_handle *h, const char *path)
{
  if (!h || !path) return DNL_ERR_ARG;
  FILE *f = fopen(path, "rb");
  if (!f) return DNL_ERR_ARG;
  std::vector<double> data;
  double buf[4096];
  size_t got;
  while ((got = fread(buf, sizeof(double), 4096, f)) > 0) data.insert(data.end(), buf, buf + got);
  fclose(f);
  const long N = h->N, nIP = dnl::ip_total(h);  // every group's points, in element order
  if (data.size() != (size_t)(6 + 1 + 6 + 1 + 23 * N + 3 + 47 * nIP + 3 + 3)) return DNL_ERR_ARG;
  In in(data);
  in.header();
  in.get();  // Structure::currentTime
  in.header();
  const double t = in.get();
  std::vector<double> x(3 * N), du(3 * N), v(3 * N), a(3 * N), disp(3 * N);
  for (long n = 0; n < N; n++) {
    double rec[23];
    in.get(rec, 23);
    for (int c = 0; c < 3; c++) {
      x[3 * n + c] = rec[c];
      v[3 * n + c] = rec[8 + c];
      a[3 * n + c] = rec[11 + c];
      du[3 * n + c] = rec[17 + c];
      disp[3 * n + c] = rec[20 + c];
    }
  }
  in.separator();
  std::vector<double> S(9 * nIP), Eps(9 * nIP), EpsPlas(9 * nIP), p(nIP), evp(nIP);
  for (long q = 0; q < nIP; q++) {
    double rec[47];
    in.get(rec, 47);
    p[q] = rec[0];
    evp[q] = rec[1];
    memcpy(&S[9 * q], rec + 2, 9 * sizeof(double));
    memcpy(&Eps[9 * q], rec + 20, 9 * sizeof(double));
    memcpy(&EpsPlas[9 * q], rec + 38, 9 * sizeof(double));
  }
  in.separator();
  in.separator();
  if (!in.ok) return DNL_ERR_ARG;
  int r;
  // the lumped mass is the one of the initial mesh (Domain::initSolve before a restart file is read)
  if (!h->prologueDone && (r = dnl_prologue(h))) return r;
  dnl_state_view sv;
  memset(&sv, 0, sizeof sv);
  sv.coords = x.data();
  sv.du = du.data();
  sv.v = v.data();
  sv.a = a.data();
  sv.disp = disp.data();
  sv.S = S.data();
  sv.Eps = Eps.data();
  sv.EpsPlas = EpsPlas.data();
  sv.p = p.data();
  sv.evp = evp.data();
  if ((r = dnl_set_state(h, &sv))) return r;
  return dnl::restart_time(h, t);
}

}  // extern "C"
