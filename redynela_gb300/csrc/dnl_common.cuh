// Shared definitions of libdnlgpu: element traits, device-side time state, kernel argument packs
// and the handle.  All arithmetic is FP64.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "dnl_gpu.h"

namespace dnl {

// ------------------------------------------------------------------------ constants
// basicTools/Math.h:36-46 (decimal literals, rounded to the nearest double like the reference)
constexpr double kPi = 3.1415926535897932384626433832795;
constexpr double kDeuxPi = 6.283185307179586476925286766559;
constexpr double kSqrt23 = 0.8164965809277260327324280249019;
constexpr double kSqrt32 = 1.2247448713915890490986420373529;
// linearAlgebra/Tensor2.C:34 and finiteElement/DefaultValues.h:24-36
constexpr double kPolarPrecision = 10.0E-10;
constexpr int kPolarMaxIt = 30;
constexpr double kRadialReturnPrecision = 1.0E-8;
constexpr int kRadialReturnMaxIt = 2000;
constexpr int kPulseMaxIt = 1000;
constexpr double kPulseConvergence = 1e-4;

// ------------------------------------------------------------------------ element traits
template <int ET> struct Elem;
template <> struct Elem<DNL_ELQUA4NAX> {
  static constexpr int DIM = 2, NEN = 4, NIP = 4;
  static constexpr int NS = 4;  // symmetric tensor components stored: xx yy zz xy
};
template <> struct Elem<DNL_ELHEX8N3D> {
  static constexpr int DIM = 3, NEN = 8, NIP = 8;
  static constexpr int NS = 6;  // xx yy zz xy xz yz
};
template <> struct Elem<DNL_ELQUA4N2D> {  // plane strain: the quad of ElQua4nAx without the hoop terms
  static constexpr int DIM = 2, NEN = 4, NIP = 4;
  static constexpr int NS = 4;
};
template <> struct Elem<DNL_ELTET4N3D> {
  static constexpr int DIM = 3, NEN = 4, NIP = 1;
  static constexpr int NS = 6;
};
template <> struct Elem<DNL_ELTET10N3D> {
  static constexpr int DIM = 3, NEN = 10, NIP = 4;
  static constexpr int NS = 6;
};
template <> struct Elem<DNL_ELHEX8N3D_1PT> {  // not a reference element (see dnl_gpu.h)
  static constexpr int DIM = 3, NEN = 8, NIP = 1;
  static constexpr int NS = 6;
};
// the same by run-time element type
__host__ __device__ constexpr bool etype_valid(int et) { return et >= DNL_ELQUA4NAX && et <= DNL_ELHEX8N3D_1PT; }
__host__ __device__ constexpr int etype_dim(int et) { return et == DNL_ELQUA4NAX || et == DNL_ELQUA4N2D ? 2 : 3; }
__host__ __device__ constexpr int etype_nen(int et)
{
  return (et == DNL_ELHEX8N3D || et == DNL_ELHEX8N3D_1PT) ? 8 : (et == DNL_ELTET10N3D ? 10 : 4);
}
__host__ __device__ constexpr int etype_nip(int et)
{
  return et == DNL_ELHEX8N3D ? 8 : ((et == DNL_ELTET4N3D || et == DNL_ELHEX8N3D_1PT) ? 1 : 4);
}
__host__ __device__ constexpr int etype_ns(int et) { return etype_dim(et) == 2 ? 4 : 6; }

// Edges of the quads and of the hexahedron along each reference axis (NE / DIM per axis, axis c
// first), as (lo, hi) local nodes with hi on the + side of the axis; lo and hi packed 4 bits per
// edge for run-time indices.  At a Gauss point the bilinear/trilinear dN/dxi_c of the two nodes of
// an edge are opposite, so sum_k dN_k/dxi_c v_k = sum over the axis-c edges of w (v_hi - v_lo),
// w the table value for the number of sign disagreements between the edge's other coordinates
// and the point's (Shape::dN).
template <int ET> struct Edges {
  static constexpr int NE = 4;  // quads: xi edges 0-1, 3-2; eta edges 0-3, 1-2
  static constexpr unsigned long long LO = 0x1030ull, HI = 0x2321ull;
};
template <> struct Edges<DNL_ELHEX8N3D> {
  static constexpr int NE = 12;  // xi: 0-1 3-2 4-5 7-6; eta: 0-3 1-2 4-7 5-6; zeta: 0-4 1-5 2-6 3-7
  static constexpr unsigned long long LO = 0x321054107430ull, HI = 0x765467236521ull;
};
__host__ __device__ constexpr int edge_node(unsigned long long packed, int e) { return (int)((packed >> (4 * e)) & 15); }

// element types with the forward-mode sensitivity path (tape and tangent kernels): all of them
__host__ __device__ constexpr bool etype_has_sens(int et) { return etype_valid(et); }
// element types whose time-step length is the quad's Courant length (else the tetrahedra's
// shortest edge; ElHex8n3D has none)
__host__ __device__ constexpr bool etype_quad(int et) { return et == DNL_ELQUA4NAX || et == DNL_ELQUA4N2D; }
// Courant length kinds: 0 the quads' (ElQua4nAx::getLength), 1 the tetrahedra's shortest edge,
// 2 the one-point hexahedron's volume / largest face area
__host__ __device__ constexpr int etype_length_kind(int et)
{
  return etype_quad(et) ? 0 : (et == DNL_ELHEX8N3D_1PT ? 2 : 1);
}

// The reference's ElTet10n3D tables (ElTet10n3D.C:45-72) as they evaluate: at Gauss point p the
// barycentric coordinate L_p is beta and the others alpha (p = 0: L0 = 1 - xi - eta - zeta), the
// shape functions are L_i (2 L_i - 1) at the corners and 4 L_i L_j at the mid-edge nodes 4..9 =
// (0,1) (1,2) (0,2) (0,3) (1,3) (2,3), and each value is one of the reference's named constants.
// Two of those constants are unparenthesised macros (1.0 - 1.0 / sqrt(5.0) and
// 1.0 + 3.0 / sqrt(5.0)); where the table negates them the expansion gives -1.0 - 1.0 / sqrt(5.0)
// and -1.0 + 3.0 / sqrt(5.0), so the derivatives -4 alpha and -4 beta are stored as those values.
inline void tet10_tables(double N[4][10], double D[4][10][3])
{
  const double r5 = sqrt(5.0);
  const double a4 = 1.0 - 1.0 / r5, b4 = 1.0 + 3.0 / r5;  // 4 alpha, 4 beta
  const double a4neg = -1.0 - 1.0 / r5, b4neg = -1.0 + 3.0 / r5;
  const double bm = 3.0 / r5, am = 1.0 / r5, ba = 4.0 / r5;  // 4 beta - 1, 1 - 4 alpha, 4 (beta - alpha)
  const int ea[6] = {0, 1, 0, 0, 1, 2}, eb[6] = {1, 2, 2, 3, 3, 3};
  for (int p = 0; p < 4; p++) {
    for (int i = 0; i < 4; i++) N[p][i] = i == p ? 0.1 : -0.1;
    for (int m = 0; m < 6; m++)
      N[p][4 + m] = (ea[m] == p || eb[m] == p) ? (1.0 + r5) / 10.0 : (3.0 - r5) / 10.0;
    for (int c = 0; c < 3; c++) {
      // corners: dN_0/dxi_c = 1 - 4 L0, dN_i/dxi_c = (4 L_i - 1) [c == i - 1]
      D[p][0][c] = p == 0 ? -bm : am;
      for (int i = 1; i < 4; i++) D[p][i][c] = c == i - 1 ? (p == i ? bm : -am) : 0.0;
      // mid-edge (a, b): 4 (L_b dL_a/dxi_c + L_a dL_b/dxi_c), dL_0/dxi_c = -1, dL_i/dxi_c = [c == i - 1]
      for (int m = 0; m < 6; m++) {
        const int A = ea[m], B = eb[m];
        const int dA = A == 0 ? -1 : (c == A - 1), dB = c == B - 1;
        double v;
        if (dA == 0 && dB == 0) {
          v = 0.0;
        } else if (dA == -1 && dB == 1) {  // 4 (L0 - L_b)
          v = p == 0 ? ba : (p == B ? -ba : 0.0);
        } else if (dA == -1) {  // -4 L_b
          v = p == B ? b4neg : a4neg;
        } else {  // 4 L_b (dA) or 4 L_a (dB)
          const int other = dA ? B : A;
          v = p == other ? b4 : a4;
        }
        D[p][4 + m][c] = v;
      }
    }
  }
}

// integration-point state, component-major: ip[comp * nIP + (e * NIP + pt)]
//   S[NS] | Eps[NS] | EpsPlas[NS] | p | evp | evpn (= evp^n, cached yield term)
template <int ET> struct IpLayout {
  static constexpr int NS = Elem<ET>::NS;
  static constexpr int S = 0, EPS = NS, EPSP = 2 * NS, P = 3 * NS, EVP = 3 * NS + 1,
                       EVPN = 3 * NS + 2, NCOMP = 3 * NS + 3;
};

// Per-integration-point record of the element pass that the tangent pass (forward-mode
// sensitivities) reads back, component-major [slot][E*NIP].  Symmetric 3x3 matrices are stored
// as xx yy zz xy xz yz.  Besides the primal quantities it holds the direction-independent
// factors of the tangent, formed once per point instead of once per parameter: the divided
// differences of ln(l)/2 and l^-1/2 over the eigenvalues of C, U^-1, and G_u = sum_k du_k dN/dxi_k.
template <int ET> struct TapeLayout {
  static constexpr int DIM = Elem<ET>::DIM, NS = Elem<ET>::NS;
  static constexpr int JI = 0;              // J^-1 [l][c], DIM x DIM
  static constexpr int DETJ = JI + DIM * DIM;
  static constexpr int RAD = DETJ + 1;      // axisymmetric radius of the Gauss point
  static constexpr int VRR = RAD + 1;       // axisymmetric (sum N_k du_k,r) / radius
  static constexpr int F = VRR + 1;         // F [r][c], 3 x 3
  static constexpr int GU = F + 9;          // G_u [r][l] = sum_k du_k[r] dN_k/dxi_l, DIM x DIM
  static constexpr int V = GU + DIM * DIM;  // eigenvectors of C = F^T F (columns), 3 x 3
  static constexpr int GD = V + 9;          // divided differences of ln(l)/2, symmetric
  static constexpr int HD = GD + 6;         // divided differences of l^-1/2, symmetric
  static constexpr int UI = HD + 6;         // U^-1 = C^-1/2, symmetric
  static constexpr int R = UI + 6;          // rotation, 3 x 3
  static constexpr int STR = R + 9;         // trial deviator (symmetric components)
  static constexpr int NORMS = STR + NS;    // its norm
  static constexpr int GAM = NORMS + 1;     // plastic multiplier (0: elastic step)
  static constexpr int XV = GAM + 1;        // evp + sqrt(2/3) gamma
  static constexpr int XN = XV + 1;         // XV^n
  static constexpr int LXV = XN + 1;        // ln XV (plastic points; the n-derivative of XV^n)
  static constexpr int NT = LXV + 1;
};

// Tangent integration-point state per parameter direction: [dir][comp][E*NIP]
template <int ET> struct TanLayout {
  static constexpr int NS = Elem<ET>::NS;
  static constexpr int S = 0, EPS = NS, EPSP = 2 * NS, P = 3 * NS, EVP = 3 * NS + 1, NCOMP = 3 * NS + 2;
};
constexpr int kSensParams = 4;  // A, B, n, |v0|

// ------------------------------------------------------------------------ device time state
// Mirrors the Solver / Domain members that drive ExplicitSolverCH::solve.
struct DevTime {
  double timeStep, currentTime, nextTime, upTime, endTime, startTime;
  double computedTimeStep, lastTimeStep, tsDate, lastTsDate;
  double kinetic;
  double fmax;                       // Pulse: sqrt of the converged eigenvalue estimate
  double fmax0;                      // Pulse: Domain::fmax0, last estimate (0 = not started)
  double pulseScale;                 // Pulse: divisor that normalises the stored vector
  unsigned long long pulseMaxBits;   // Pulse: max |M^-1 K x| of the running iteration
  unsigned long long lenMinBits;     // Courant: min element length (bits of a positive double)
  long long increment;
  long long pulseTotal;              // Pulse: power iterations over the run
  int done;
  int status;
  int badElem;
  int pulseDone;                     // Pulse: power iteration converged
  int pulseIter;                     // Pulse: iterations of the running call
  int pad;
};

// ------------------------------------------------------------------------ kernel arguments
// The isotropic hardening attached to a material (DNL_HARD_*), passed by value to the non-power
// laws' evaluation.
struct HardLaw {
  int law;
  int tabN;          // tabular law: number of points, abscissae tab[0..N), ordinates tab[N..2N)
  const double *tab; // device
  double P[8];       // Metafor law: P1..P8
};

struct Material {
  double young, nu, rho, A, B, n;
  double K;          // bulk modulus E / (3 (1 - 2 nu))            (Element.C:232)
  double G2, G3;     // 2 G and 3 G with G = E / (2 (1 + nu))      (Material.h:167-172)
  double nB;         // n B
  double dfun0;      // Sqrt32 * 2.0 * G, first term of dfun      (Element.C:309)
  double Cs;         // Courant sound speed with the mean nodal density (Element.C:607-621)
  double rG3;        // 1 / (3 G), for the first radial-return guess (Element.C:298)
  HardLaw hard;
};

// Material constants from the ABI description, in the reference's expressions.
#include <math.h>
inline Material make_material(const dnl_material &mt, int nen = 4)
{
  Material m;
  m.young = mt.young;
  m.nu = mt.poisson;
  m.rho = mt.density;
  m.A = mt.A;
  m.B = mt.B;
  m.n = mt.n;
  m.K = m.young / (3. * (1. - 2. * m.nu));
  const double G = m.young / (2. * (1. + m.nu));
  m.G2 = 2.0 * G;
  m.G3 = 3.0 * G;
  m.nB = m.n * m.B;
  m.dfun0 = kSqrt32 * 2.0 * G;
  m.rG3 = 1.0 / m.G3;
  // Element::getSoundSpeed uses the mean of the element's nodal densities
  double ro = 0.;
  for (int i = 0; i < nen; i++) ro += m.rho;
  ro /= nen;
  const double Nu = m.nu;
  m.Cs = sqrt((m.young * (1 - Nu)) / (ro * (1 + Nu) * (1 - 2 * Nu)));
  m.hard.law = DNL_HARD_POWER;
  m.hard.tabN = 0;
  m.hard.tab = nullptr;
  for (int k = 0; k < 8; k++) m.hard.P[k] = 0.;
  return m;
}

// A material with any of the hardening laws (the moduli as make_material; power-law parameters
// from params[0..2]; the tabular law's table already on the device at `tab`).
inline Material make_material_law(const dnl_material_law &ml, const double *tab)
{
  dnl_material mt;
  mt.young = ml.young;
  mt.poisson = ml.poisson;
  mt.density = ml.density;
  const bool power = ml.law == DNL_HARD_POWER;
  mt.A = power ? ml.params[0] : 0.;
  mt.B = power ? ml.params[1] : 0.;
  mt.n = power ? ml.params[2] : 0.;
  Material m = make_material(mt);
  m.hard.law = ml.law;
  m.hard.tabN = ml.law == DNL_HARD_TABULAR ? ml.npoints : 0;
  m.hard.tab = tab;
  for (int k = 0; k < 8; k++) m.hard.P[k] = ml.params[k];
  return m;
}

struct NodeFields {  // one NodalField bank, SoA, 3 components each
  double *du[3], *v[3], *a[3], *disp[3];
};

struct ElemArgs {
  int E, N;
  int gate;            // 1: skip the pass once the run is done or an error is recorded
  const int *conn;     // [NEN][E]
  double *x[3];        // current coordinates
  const double *du[3]; // Current delta_disp
  const double *v[3];  // Current mat_speed (the one-point hexahedron's hourglass viscosity)
  double hourglass;    // its coefficient
  double *ip;          // integration-point state
  double *fe;          // element forces: component i of element e's node k at fe[i feStride + e NEN + k]
  long feStride;       // element-node slots of the handle's element groups (E*NEN with one type)
  int eBase;           // the domain's number of element 0 of these arguments (error reports)
  double *detJ;        // [E*NIP] (written)
  double *stepT;       // optional dEps|R per IP, [18][E*NIP] or nullptr
  double *tape;        // [TapeLayout::NT][E*NIP], written by the tape instance of k_elem
  DevTime *tm;
  Material mat;
  const int *elemMat;       // several materials: material of each element (mats), or nullptr
  const Material *mats;
  const double *elemCs;     // several materials: Courant sound speed of each element
};

// Tangent element pass: the primal pass's inputs and record, the tangents of its inputs
// (coordinates and Current delta_disp, [dir][3][N]) and of the integration-point state.
struct SensElemArgs {
  int E, N;
  const int *conn;
  const double *x[3];
  const double *du[3];
  const double *ip;    // integration-point state after the primal pass
  const double *tape;  // [TapeLayout::NT][E*NIP]
  const double *tx;    // [dir][3][N]
  const double *tdu;   // [dir][3][N]
  const double *v[3];  // Current velocities (the one-point hexahedron's hourglass force)
  const double *tv;    // their tangents, [dir][3][N]
  double hourglass;    // its coefficient
  double *tip;         // [dir][TanLayout::NCOMP][E*NIP]
  double *tfe;         // [dir][DIM][feStride]: the element's slots from e NEN
  long feStride;       // element-node slots of the handle's element groups (E*NEN with one type)
  DevTime *tm;
  Material mat;
  const int *elemInst; // batched: instance of each element (its material), or nullptr
  const Material *mats;
};

// Adjoint (reverse mode) of the element pass: the pass's record and output state, the adjoints of
// its outputs, and where the adjoints of its inputs go (dnl_adj_elem.cuh).
struct AdjElemArgs {
  int E, N;
  const int *conn;        // [NEN][E]
  const double *x[3];     // coordinates the pass read
  const double *tape;     // [TapeLayout::NT][E*NIP], written by the tape instance of k_elem
  const double *ipOut;    // integration-point state after the pass [IpLayout::NCOMP][E*NIP]
  const double *fbar;     // adjoint of the assembled nodal forces, [3][N]
  double *ipAdj;          // [TanLayout::NCOMP][E*NIP]: in, adjoint of the state after the pass;
                          // out, of the state before it
  double *xe, *ue;        // [DIM][feStride]: adjoints of the element nodes' coordinates and
                          // Current delta_disp from this pass (the element's slots from e NEN)
  long feStride;          // element-node slots of the handle's element groups (E*NEN with one type)
  double *gpar;           // [3][gStride]: d L / d(A, B, n) accumulated per integration point
  long gStride;           // integration points of the handle's element groups (E*NIP with one type)
  Material mat;
};

struct GatherArgs {
  int N, EN;              // EN = E*NEN
  const int *start;       // node -> CSR offsets, N+1
  const int *entry;       // entries e*NEN+k, ascending e within a node
  const double *fe;       // [DIM][EN]
  double *fint;           // [N*DIM], Id*dim+j
};

struct NodeArgs {
  int N, EN;
  const int *start, *entry;
  const double *fe;
  const double *mass;
  NodeFields cur, nxt;
  double *x[3];
  const int *bcIdx;       // per node: -1 or index into bcCode/bcSpeed
  const int *bcCode;      // 2 bits per component: 0 none, 1 restrained, 2 imposed speed
  const double *bcSpeed;  // 3 per BC node
  double *fint;           // optional [N*DIM] copy of the assembled forces
  DevTime *tm;
  double alphaM, beta, gamma;
};

// per-instance constants of a batch
struct InstParams {
  double alphaM, beta, gamma, safetyOmega, Cs;
  int freq, method;
};

// One batched explicit step as a single persistent (cooperative) launch: the phases of the
// launch sequence -- time logic, boundary conditions, element pass, nodal update, Courant
// reduction when due, time logic -- separated by grid-wide barriers (dnl_elem.cu).
struct BatchStepArgs {
  ElemArgs ea;              // the union mesh; du / v of the Current bank
  NodeArgs na;              // nodal update Current -> New (tm unused: per-instance records)
  NodeFields cur;           // Current bank, for the boundary-condition writes
  const int *elemInst, *nodeInst;
  const Material *mats;
  const InstParams *prm;
  DevTime *tms;
  int count;
  int nbc;                  // boundary-condition nodes
  const int *bcNodes;
  int preFirst;             // 1: the time logic's initStep (DT_PRE) opens the step
  int courant;              // 1: the Courant lengths are due after the nodal update
  int postMode;             // DT_POST, or DT_POST | DT_PRE when another step follows
  unsigned *bar;            // barrier: arrival count, generation
  int *err;                 // 1 when a barrier wait ran out (DNL_ERR_TIMEOUT)
};

// ------------------------------------------------------------------------ handle
struct GraphEntry {
  int nsteps, parity, phase;
  cudaGraphExec_t exec;
};

}  // namespace dnl

namespace dnl {
// A further group of elements of another type in the same domain (dnl_add_elements): its elements
// are numbered after those of the handle's first group and of the groups added before it.  Its
// element-node slots in fe / kx / the lumped-mass vector start at feOff.
struct ElemGroup {
  int etype, nen, nip, E;
  int eOff;      // the domain's number of the group's first element
  long nIP, feOff;
  long ipOff;    // the group's first integration point in element order (its state is the block
                 // at ip + NCOMP ipOff of the handle's one integration-point allocation)
  int *conn;     // [NEN][E]
  double *ip;    // integration-point state [NCOMP][nIP], inside the handle's allocation
  double *detJ;  // [nIP]
  double *pj;    // Pulse per-Gauss-point kinematics, or nullptr
  double *Cs;    // Courant: the sound speed of each element when the groups' differ, or nullptr
  double *stepT; // dEps|R per IP [18][nIP] when the handle keeps them, or nullptr
};
}  // namespace dnl

struct dnl_handle {
  int etype, dim, nen, nip, N, E, nIP;  // the first element group (the only one unless
                                         // dnl_add_elements added others)
  int flags;
  cudaStream_t stream;
  // mesh
  int *conn;                  // [NEN][E]
  double *x[3];
  int *n2eStart, *n2e;        // node -> element entries
  double *mass;               // N
  // nodal fields, two banks (Node::Current / Node::New swap by index)
  double *fieldMem;
  dnl::NodeFields bank[2];
  int cur;
  // integration points
  double *ip;
  double *detJ;
  double *stepT;
  double *fe;                 // [DIM][EN]
  long EN;                    // element-node slots of all element groups
  int nextra;                 // further element groups (dnl_add_elements)
  dnl::ElemGroup *extra;
  bool batchUnion;            // the union mesh of a dnl_batch
  double *fint;               // [N*DIM]
  // boundary conditions
  int nbcNodes;
  int *bcIdx, *bcCode, *bcNodeList;
  double *bcSpeed;
  bool hasSpeedBC;
  // Pulse: per Gauss point J^-1, weight x detJ (x 2 pi R) and R; the iterated vector (raw)
  double *pj, *ev, *kx;
  double C00, C01, C33;       // Hooke matrix entries (Material::getHookeMatrix)
  double hourglass;           // DNL_ELHEX8N3D_1PT: viscous hourglass coefficient (0.05)
  // time
  dnl::DevTime *tm;
  dnl::Material mat;
  double alphaM, beta, gamma, omegaS, safetyOmega;
  double endTime, rhoB, safety;
  int freq, method;
  bool prologueDone;
  long long hostIncrement;    // host copy of tm->increment, valid between calls
  // graphs
  dnl::GraphEntry graphs[8];
  int ngraphs;
  char lastError[256];
  double *stage;              // 5 x N*3 staging buffer for host <-> device nodal vectors (one
                              // slot per nodal field, so the copies of a call run back to back)
  cudaEvent_t marks[8];
  // dnl_step_host: the second stream its transfers run on, its events, the boundary conditions'
  // device flag (created on first use)
  cudaStream_t ioStream;
  cudaEvent_t ioEv[3];
  int *bcApplied;
  // per-kernel event timing (dnl_profile_begin/end)
  bool profiling;
  void *prof;
  // several materials (dnl_set_materials)
  int nmat;
  int *elemMat;               // device, E, or nullptr (one material: mat)
  dnl::Material *dmats;       // device, nmat
  double *elemCs;             // device, E: sound speed with the nodal densities of Domain::initSolve
  double *matTab;             // device: the tabular laws' points
  double *evpn0;              // device, nmat: (1e-10)^n of power-law materials (dnl_reset)
  double *hooke;              // device, nmat x 3: each material's Hooke entries C00, C01, C33 for
                              // the Pulse products, with several materials and the Pulse step
  double *nodeRo;             // host, N: Current ro of the first nodal field (results files)
  // several materials, host copies: each element's material (every group, element order) and
  // each material's power-law exponent (0 for the other laws), for the cached evp^n of
  // dnl_set_state
  int *elemMatHost;
  double *matExpHost;
  // initial state (dnl_reset)
  double *x0;                 // initial coordinates [3][N]
  double v0[3];               // initial velocity
  // forward-mode sensitivities (dnl_sens.cu)
  double v0dir[3];            // unit vector of the initial velocity
  void *sens;
  // reverse-mode adjoint: checkpoints, step records and adjoint state (dnl_adjoint.cu)
  void *adj;
};

namespace dnl {
// integration points of every element group, in element order (the first group's, then each
// added group's)
inline long ip_total(const dnl_handle *h)
{
  long n = h->nIP;
  for (int gi = 0; gi < h->nextra; gi++) n += h->extra[gi].nIP;
  return n;
}
}  // namespace dnl

// 1/x by the Newton-Raphson iteration for the reciprocal (the root of f(r) = 1/r - x: r <- r (2 - x r),
// written r + r e with the residual e = 1 - x r in one fused multiply-add; the relative error
// squares at each step), started from the PTX hardware seed rcp.approx.ftz.f64.  Two steps give the
// double result within one ulp of the IEEE quotient 1.0 / x (the bound the self-check test holds;
// on 1,049,194 random and edge inputs across the domain, dnl_check_quotients measured it equal to
// CUDA's IEEE division every time).
// Domain: normal finite x with 2^-1022 < |x| < 2^1022.  The seed flushes subnormals (.ftz), so a
// subnormal x, or an x whose reciprocal is subnormal (|x| > 2^1022), gives inf or 0 instead of
// the IEEE result.  Every call site passes a positive normal quantity well inside that range
// (Gauss-point radius, lumped nodal mass, evp >= 1e-10, the Newton derivative, 1 - alphaM).
__device__ __forceinline__ double nr_rcp(double x)
{
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}

// a / b from r = nr_rcp(b) and one residual correction (q0 = a r, q = q0 + (a - q0 b) r; Markstein's
// sequence): the correctly rounded quotient but in rare hard cases (within one ulp; equal to the
// IEEE quotient on the same 1,049,194 inputs), 3 FP64
// instructions where an IEEE division takes 17.  Same domain for b as nr_rcp; a / b must be normal.
__device__ __forceinline__ double quot(double a, double b, double r)
{
  const double q0 = a * r;
  return fma(fma(-q0, b, a), r, q0);
}

// CALL instantiated for the handle's element type, as ET (CALL in parentheses when it has commas)
#define DNL_ET_CASE(etype, T, CALL) \
  if ((etype) == (T)) {             \
    constexpr int ET = (T);         \
    CALL;                           \
  }
#define DNL_BY_ETYPE(etype, CALL)                                           \
  do {                                                                      \
    DNL_ET_CASE(etype, DNL_ELQUA4NAX, CALL)                                 \
    else DNL_ET_CASE(etype, DNL_ELQUA4N2D, CALL)                            \
    else DNL_ET_CASE(etype, DNL_ELHEX8N3D_1PT, CALL)                        \
    else DNL_ET_CASE(etype, DNL_ELTET4N3D, CALL)                            \
    else DNL_ET_CASE(etype, DNL_ELTET10N3D, CALL)                           \
    else {                                                                  \
      constexpr int ET = DNL_ELHEX8N3D;                                     \
      CALL;                                                                 \
    }                                                                       \
  } while (0)

namespace dnl {
// launchers implemented in dnl_elem.cu
int launch_elem(dnl_handle *h, cudaStream_t s, int gate);
int launch_elem_tape(dnl_handle *h, cudaStream_t s, double *tape);
int launch_elem_tan(int etype, const SensElemArgs &a, cudaStream_t s);
int launch_elem_batch_tape(int etype, const ElemArgs &a, const int *elemInst, const Material *mats,
                           DevTime *tms, cudaStream_t s);
// batched instance tables for the sensitivity run (nullptr members: a single mesh)
struct SensBatch {
  int count;
  const int *elemInst, *nodeInst;
  const Material *mats;
  const InstParams *prm;
  DevTime *tms;
  const double *v0dir;  // [count][3]
};
int sens_run(dnl_handle *h, int nsteps, const double *dts, const SensBatch *bt);
// reverse mode (dnl_adjoint.cu, dnl_adj_elem.cuh)
int launch_elem_adj(int etype, const AdjElemArgs &a, cudaStream_t s);
int launch_elem_tape_raw(int etype, const ElemArgs &a, cudaStream_t s);
void adj_free(dnl_handle *h);
int adjoint_forward(dnl_handle *h, const double *dts, int nsteps, int stride);
int adjoint_backward(dnl_handle *h, const double *dL_dx, double *grad, dnl_adjoint_info *info);
int sens_schedule(dnl_handle *h, const double **dts, int *n);
int sens_outputs(dnl_handle *h, double *coords, double *dcoords);
void sens_free(dnl_handle *h);
// primal per-step launches (dnl_host.cu) used by the sensitivity run
int enqueue_bc_current(dnl_handle *h);
int enqueue_node(dnl_handle *h);
int read_time_state(dnl_handle *h, DevTime *t);
int restart_time(dnl_handle *h, double t);
int launch_mass(dnl_handle *h, cudaStream_t s, double *me);
int launch_courant(dnl_handle *h, cudaStream_t s);
int launch_pulse(dnl_handle *h, cudaStream_t s);
void set_shape_tables();
// loop limits of the element pass (Jacobi passes, Newton iterations; device constants of the
// current device) and of the Pulse power iteration (host-side)
int set_iteration_caps(int rotations, int newton);
int set_stop_tolerances(double polar, double radial);
int &pulse_cap();
long long &launch_counter();
// batched launches (dnl_batch.cu)
int launch_elem_batch(int etype, int block, const ElemArgs &a, const int *elemInst,
                      const Material *mats, DevTime *tms, cudaStream_t s);
int launch_mass_batch(int etype, const ElemArgs &a, double *me, const int *elemInst,
                      const Material *mats, cudaStream_t s);
int launch_courant_batch(int etype, const ElemArgs &a, const int *elemInst, DevTime *tms,
                         cudaStream_t s);
// one batched step as a persistent cooperative launch (ElQua4nAx); grid from the occupancy
int launch_batch_persistent(int etype, int block, const BatchStepArgs &a, cudaStream_t s);
ElemArgs elem_args_of(dnl_handle *h);
// the element pass's arguments for element group gi (-1: the first group, as elem_args_of)
ElemArgs group_args_of(dnl_handle *h, int gi);
int launch_node_batch(dnl_handle *h, const int *nodeInst, const InstParams *prm, DevTime *tms);
int launch_dt_batch(dnl_handle *h, DevTime *tms, const InstParams *prm, int count, int mode);
int launch_bc_batch(dnl_handle *h, DevTime *tms, const int *nodeInst);
int launch_gather_mass(dnl_handle *h, const double *me);
// launches on caller-built arguments (no handle)
int launch_elem_raw(int etype, const ElemArgs &a, cudaStream_t s);
int launch_gather_raw(int dim, const GatherArgs &g, cudaStream_t s);
// event brackets around one launch when the handle is profiling
void prof_begin(dnl_handle *h, cudaStream_t s);
void prof_end(dnl_handle *h, int kind, cudaStream_t s);
}  // namespace dnl
