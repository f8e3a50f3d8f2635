/*
 * libmgpbd.so: the comparison solvers of the MGPBD convergence experiments
 * (experiments/exp_convergence.py:26-57,119-145) and the greedy colourings
 * they run on.
 *
 *   - local XPBD, one coupled hydrostatic + deviatoric constraint per tet:
 *     the reference's `Deform3D` (cons/deform3d.py:7-288), a `pbd_framework`
 *     constraint (init_rest_status / preupdate_cons / update_cons);
 *   - Vertex Block Descent: the reference's `VBDSolver` (cons/vbd.py:6-361),
 *     a stepper like MGPBDSolverGPU (init / make_prediction / solve /
 *     update_vel / step);
 *   - greedy element and vertex colourings (utils/graph_coloring.py:24-191).
 *
 * Conventions are those of mgpbd.h: 0 or a negative MGPBD_E* code, no
 * exceptions across the ABI, mgpbd_last_error() for the text.  Mesh arrays
 * are caller-owned DEVICE pointers that must outlive the handle (the
 * solvers keep them, like the reference keeps its Taichi fields); the
 * colouring entry points take HOST arrays.
 */
#ifndef MGPBD_LOCAL_H_
#define MGPBD_LOCAL_H_

#include <stdint.h>

#include "mgpbd.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- greedy colourings (host) ------------------------------------------ */

/* color_elements (utils/graph_coloring.py:126-141): elements conflict when
 * they share a vertex.  elems: n_elements * verts_per_element vertex ids.
 * ordered: n_elements slots; offsets: n_elements + 1 slots (n_colors + 1
 * used).  Returns MGPBD_EINVAL for an id outside [0, n_vertices). */
int mgpbd_color_elements(const int32_t* elems, int32_t n_elements, int32_t verts_per_element,
                         int32_t n_vertices, int32_t* ordered, int32_t* offsets,
                         int32_t* n_colors);
/* color_vertices (:144-159): vertices conflict when they share an element.
 * ordered: n_vertices slots; offsets: n_vertices + 1 slots. */
int mgpbd_color_vertices(const int32_t* elems, int32_t n_elements, int32_t verts_per_element,
                         int32_t n_vertices, int32_t* ordered, int32_t* offsets,
                         int32_t* n_colors);
/* greedy_coloring (:78-103) over an explicit adjacency in CSR form
 * (adj_ptr: n + 1, adj: neighbour ids); ordered: n, offsets: n + 1. */
int mgpbd_greedy_coloring(const int32_t* adj_ptr, const int32_t* adj, int32_t n,
                          int32_t* ordered, int32_t* offsets, int32_t* n_colors);

/* ---- local XPBD (Deform3D) --------------------------------------------- */

#define MGPBD_XPBD_DEFAULT 0        /* all tets at once, atomic position adds
                                       (solve_cons, cons/deform3d.py:55-127)  */
#define MGPBD_XPBD_GAUSS_SEIDEL 1   /* tets one at a time in index order
                                       (solve_cons_gauss_seidel, :128-200)    */
#define MGPBD_XPBD_GRAPH_COLORING 2 /* colour by colour, the tets of a colour
                                       at once (solve_cons_graph_coloring and
                                       solve_range, :210-288)                 */

typedef struct mgpbd_xpbd_params {
  float dt;          /* substep length                                       */
  float hydro_alpha; /* compliance of det F - 1      (Deform3D.hydro_alpha)  */
  float devia_alpha; /* compliance of |F|^2 - 3      (Deform3D.devia_alpha)  */
  int32_t method;    /* MGPBD_XPBD_*                                         */
} mgpbd_xpbd_params;

typedef struct mgpbd_xpbd* mgpbd_xpbd_handle;

/* Deform3D.__init__ (cons/deform3d.py:9-35) */
int mgpbd_xpbd_create(const mgpbd_xpbd_params* params, mgpbd_xpbd_handle* out);
void mgpbd_xpbd_destroy(mgpbd_xpbd_handle h);
int mgpbd_xpbd_set_stream(mgpbd_xpbd_handle h, void* stream);
/* the mesh fields v_p (x, nv x 3, updated in place), v_p_ref (nv x 3),
 * v_invm (nv), t_i (4 nt) and t_m (nt); the graph colouring method colours
 * the tets here (compute_graph_coloring, :202-208) */
int mgpbd_xpbd_set_mesh(mgpbd_xpbd_handle h, float* x, const float* x_ref, const float* invm,
                        const int32_t* t_i, const float* t_m, int32_t nv, int32_t nt);
/* preupdate_cons (:40-42): both multipliers to zero */
int mgpbd_xpbd_preupdate(mgpbd_xpbd_handle h);
/* update_cons (:44-52), n_passes times.  Asynchronous on the handle's
 * stream; a grid barrier of the colour kernel that gave up is reported by a
 * later call, or by mgpbd_xpbd_synchronize. */
int mgpbd_xpbd_update(mgpbd_xpbd_handle h, int32_t n_passes);
/* waits for the last update and reports its status */
int mgpbd_xpbd_synchronize(mgpbd_xpbd_handle h);
/* device pointers of hydro_lambda / devia_lambda (nt each) */
int mgpbd_xpbd_lambdas(mgpbd_xpbd_handle h, float** hydro, float** devia);
/* colours of the graph colouring method (0 for the other methods) */
int mgpbd_xpbd_n_colors(mgpbd_xpbd_handle h, int32_t* n_colors);

/* ---- Vertex Block Descent (VBDSolver) ---------------------------------- */

#define MGPBD_VBD_SERIAL 0 /* vertices one at a time in index order
                              (_solve_all_serial, cons/vbd.py:185-266)        */
#define MGPBD_VBD_COLOR 1  /* colour by colour, the vertices of a colour at
                              once (_solve_vertex_range, :267-361)            */

typedef struct mgpbd_vbd_params {
  float dt;
  float damp;            /* velocity damping of update_vel                   */
  float youngs_modulus;  /* E; mu = E / (2 (1 + nu)), lambda = E nu / ((1 + nu)(1 - 2 nu)) */
  float poissons_ratio;  /* nu                                                */
  float damping;         /* Rayleigh-style damping coefficient kd             */
  float rho;             /* Chebyshev spectral-radius estimate (0 = off)      */
  float gravity[3];
  int32_t n_iterations;
  int32_t method;        /* MGPBD_VBD_*                                       */
} mgpbd_vbd_params;

typedef struct mgpbd_vbd* mgpbd_vbd_handle;

/* VBDSolver.__init__ (cons/vbd.py:9-66) and its vertex-tet adjacency
 * (_build_vertex_tet_adjacency, :68-96) */
int mgpbd_vbd_create(const mgpbd_vbd_params* params, mgpbd_vbd_handle* out);
void mgpbd_vbd_destroy(mgpbd_vbd_handle h);
int mgpbd_vbd_set_stream(mgpbd_vbd_handle h, void* stream);
int mgpbd_vbd_set_mesh(mgpbd_vbd_handle h, float* x, const float* x_ref, const float* invm,
                       const int32_t* t_i, int32_t nv, int32_t nt);
/* init (:106-124): Dm_inv and rest volumes */
int mgpbd_vbd_init(mgpbd_vbd_handle h);
int mgpbd_vbd_make_prediction(mgpbd_vbd_handle h); /* :125-132 */
int mgpbd_vbd_solve(mgpbd_vbd_handle h);           /* :134-160 */
int mgpbd_vbd_update_vel(mgpbd_vbd_handle h);      /* :161-166 */
int mgpbd_vbd_step(mgpbd_vbd_handle h);            /* :168-172 */
/* waits for the last solve and reports its status (solve, like update
 * above, is asynchronous on the handle's stream) */
int mgpbd_vbd_synchronize(mgpbd_vbd_handle h);
/* the omega of each iteration of solve (n_iterations values, 1 where the
 * Chebyshev step is off), as the reference records it */
int mgpbd_vbd_omegas(mgpbd_vbd_handle h, float* omegas);
/* device pointers of the solver-owned fields */
#define MGPBD_VBD_FIELD_V 0       /* (nv,3) v_v                                */
#define MGPBD_VBD_FIELD_X_OLD 1   /* (nv,3) v_p_old                            */
#define MGPBD_VBD_FIELD_X_TILDE 2 /* (nv,3) x_tilde                            */
#define MGPBD_VBD_FIELD_DM_INV 3  /* (nt,3,3) Dm_inv                           */
#define MGPBD_VBD_FIELD_REST_VOL 4 /* (nt) rest_vol                            */
int mgpbd_vbd_field(mgpbd_vbd_handle h, int32_t field, void** dev_ptr, int64_t* count);
int mgpbd_vbd_n_colors(mgpbd_vbd_handle h, int32_t* n_colors);
int mgpbd_vbd_lame(mgpbd_vbd_handle h, float* mu, float* lam);

#ifdef __cplusplus
}
#endif

#endif /* MGPBD_LOCAL_H_ */
