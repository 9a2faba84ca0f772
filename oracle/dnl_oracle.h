/* CPU restatement of DynELA's explicit step -- the ORACLE (test infrastructure only).
 *
 * Only tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this library, and
 * only as the checker / the timed CPU baseline.  The product path (libdnlgpu.so) never calls it.
 *
 * Element types: ElQua4nAx (etype 0, 4 nodes, 2x2 Gauss points), ElHex8n3D (etype 1, 8 nodes,
 * 2x2x2 Gauss points) and ElQua4n2D (etype 2, plane strain, the tables of ElQua4nAx).  Storage mirrors the reference objects: nodal vectors are (N, 3) like Vec3D,
 * integration-point tensors are (E, nip, 3, 3) row-major like Tensor2 (linearAlgebra/Tensor2.h).
 */
#ifndef DNL_ORACLE_H
#define DNL_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dnlo dnlo;

enum {
  DNLO_OK = 0,
  DNLO_ERR_NEG_DETJ = 1,     /* Element2D.C:101-109 (2D aborts; 3D only reports, Element3D.C:98-105) */
  DNLO_ERR_RR_NOCONV = 2,    /* Element.C:327-330, more than 2000 Newton iterations */
  DNLO_ERR_JACOBI_NOCONV = 3,/* Tensor2.C:1257-1258, 29 Jacobi sweeps without convergence */
  DNLO_ERR_PULSE_NOCONV = 4, /* Domain.C:936-939, more than 1000 power iterations */
  DNLO_ERR_DT = 5,           /* non-positive or non-finite time step */
  DNLO_ERR_ARG = 6,
  DNLO_ERR_SINGULAR = 7      /* Matrix.C:1680-1690, exactly singular Jacobian */
};

/* hardening laws: IsoHardElastoplastic, none (Material::isYield false), IsoHardElastoplasticTabular,
 * IsoHardMetafor */
enum { DNLO_HARD_POWER = 0, DNLO_HARD_ELASTIC = 1, DNLO_HARD_TABULAR = 2, DNLO_HARD_METAFOR = 3 };

/* solver[5] = {tend, rho_b, safety, freq, method (0 Courant, 1 Pulse)}
 * mat[6]    = {E, nu, rho, A, B, n}
 * BC groups: kind 0 = BoundaryRestrain (val = 0/1 mask), 1 = BoundarySpeed (val = velocity);
 * group g covers bc_nodes[bc_start[g] .. bc_start[g+1]). */
dnlo *dnlo_create(int etype, long N, long E, const double *coords, const long *conn,
                  const double *mat, const double *v0, long nbc, const long *bc_kind,
                  const double *bc_val, const long *bc_start, const long *bc_nodes,
                  const double *solver);
void dnlo_destroy(dnlo *h);

/* Direct access to the state arrays by name (see dnl_oracle.c: field table). */
double *dnlo_array(dnlo *h, const char *name, long *count);
double dnlo_get(dnlo *h, const char *name);
int dnlo_set(dnlo *h, const char *name, double value);

int dnlo_internal_matrices(dnlo *h, int reference);
int dnlo_internal_forces(dnlo *h);
int dnlo_mass(dnlo *h);
int dnlo_time_step(dnlo *h, int force);
double dnlo_courant(dnlo *h);
int dnlo_max_frequency(dnlo *h, double *fmax);
int dnlo_prologue(dnlo *h);
int dnlo_steps(dnlo *h, long nsteps, long *done);
int dnlo_bad_element(dnlo *h);
int dnlo_tables(int etype, double *N, double *dN);
void dnlo_set_threads(int n);
int dnlo_get_threads(void);
/* several materials / hardening laws (props nmat x 12: E nu rho law P1..P8), initial velocities */
int dnlo_set_materials(dnlo *h, int nmat, const double *props, const long *tab_start,
                       const double *tab_x, const double *tab_y, const long *elem_mat);
int dnlo_set_velocity(dnlo *h, const double *v);
/* etype 5 (the one-point hexahedron, not a reference element): viscous hourglass coefficient */
int dnlo_set_hourglass(dnlo *h, double coefficient);

#ifdef __cplusplus
}
#endif
#endif
