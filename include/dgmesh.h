/*
 * dgmesh.h - C ABI of the host-side mesh layer that feeds dgcuda.h: .msh
 * reading/writing, structured simplex box generation, the reference-semantics
 * Mesh precompute and the .conf parser.
 *
 * What it replaces (reference file:line):
 *   dgm_read_msh       gmsh::open + gmsh::model::mesh::getElementsByType
 *                      (src/dgalerkin.cpp:24-26, src/Mesh.cpp:25-38)
 *   dgm_precompute     the Mesh constructor (src/Mesh.cpp:20-435) with
 *                      getUniqueFaceNodeTags (src/Mesh.cpp:679-713)
 *   dgm_get_desc       read access to the Mesh arrays (include/Mesh.h:31-108)
 *   dgm_parse_config   config::parseConfig (src/configParser.cpp:30-150)
 *   dgm_gaussian_ic    the initial condition loop (src/dgalerkin.cpp:37-50)
 *   dgm_source_dofs    source node selection (src/solver.cpp:197-210)
 *   dgm_box_tri/tet    no counterpart (the reference reads gmsh-made meshes)
 * Return codes are the DG_* codes of dgcuda.h; dg_last_error() has the text.
 */
#ifndef DGMESH_H
#define DGMESH_H

#include "dgcuda.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dgm_mesh dgm_mesh;
typedef struct dgm_precomp dgm_precomp;
typedef struct dgm_config dgm_config;

/* Read-only view of a raw mesh; pointers live as long as the mesh. */
typedef struct dgm_raw {
    int dim, order, el_type, np;
    int num_nodes;
    const int *node_tags;     /* [num_nodes] */
    const double *xyz;        /* [num_nodes][3] */
    int num_el;
    const int *el_tags;       /* [num_el] */
    const int *el_nodes;      /* [num_el][np] node tags, gmsh order */
    int num_phys;
    const int *phys_dim;      /* [num_phys] */
    const int *phys_tag;      /* [num_phys] */
    const char *const *phys_name;   /* [num_phys] */
    const int *phys_node_offsets;   /* [num_phys+1] */
    const int *phys_nodes;          /* node tags of each group, sorted */
} dgm_raw;

int dgm_read_msh(const char *path, dgm_mesh **out);
int dgm_write_msh(const dgm_mesh *m, const char *path);
/* side_names: {y=lo, x=hi, y=hi, x=lo}; NULL entries leave a side unnamed. */
int dgm_box_tri(int nx, int ny, const double lo[2], const double hi[2], int order,
                const char *const side_names[4], dgm_mesh **out);
/* side_names: {x=lo, x=hi, y=lo, y=hi, z=lo, z=hi}; removed cells are
 * i + nx*(j + ny*k); their faces form the obstacle_name group. */
int dgm_box_tet(int nx, int ny, int nz, const double lo[3], const double hi[3], int order,
                const char *const side_names[6], const int *removed, int nremoved,
                const char *obstacle_name, dgm_mesh **out);
int dgm_get_raw(const dgm_mesh *m, dgm_raw *out);
/* Replace the coordinates of every node (xyz[num_nodes][3], in the order of
 * dgm_raw.node_tags), e.g. to curve a generated mesh; no counterpart in the
 * reference, which reads node positions from gmsh. */
int dgm_set_nodes(dgm_mesh *m, const double *xyz);
void dgm_free_mesh(dgm_mesh *m);

/* Boundary conditions: physical tags (dimension dim-1) in ascending order,
 * reflecting (1) or absorbing (0). */
int dgm_precompute(const dgm_mesh *m, int nbc, const int *bc_phys_tags, const int *bc_reflecting,
                   dgm_precomp **out);
int dgm_get_desc(const dgm_precomp *p, dg_mesh_desc *out);
/* Number of curved (non-affine) elements and a per-element flag [num_el]. */
int dgm_get_curved(const dgm_precomp *p, int *ncurved, const unsigned char **flags);
int dgm_get_dof_coords(const dgm_precomp *p, const double **xyz); /* [num_el*np][3] */
int dgm_get_face_node_tags(const dgm_precomp *p, const int **tags); /* [f_num][f_num_nodes] */
double dgm_min_edge(const dgm_precomp *p);
void dgm_free_precomp(dgm_precomp *p);

/* u0[num_el*np] += amp*exp(-|x-x0|^2/size) over every element node. */
int dgm_gaussian_ic(const dgm_precomp *p, double x, double y, double z, double size, double amp, double *u0);
/* Element-node indices with |x-xs|^2 < size^2; *count = number found (may
 * exceed cap, in which case only cap are written). */
int dgm_source_dofs(const dgm_precomp *p, double x, double y, double z, double size, int *idx, int cap,
                    int *count);

typedef struct dgm_config_view {
    double time_start, time_end, time_step, time_rate;
    int num_threads;
    double v0[3];
    double rho0, c0;
    int num_sources;
    const double *sources;    /* [num_sources][9]: pole,x,y,z,size,amp,freq,phase,duration */
    int num_ics;
    const double *ics;        /* [num_ics][6]: 0,x,y,z,size,amp */
    int num_bcs;
    const int *bc_phys_tags;  /* ascending */
    const int *bc_reflecting;
    const char *element_type, *time_int_method, *save_file, *precision, *flux_sign;
} dgm_config_view;

int dgm_parse_config(const char *path, const dgm_mesh *m, dgm_config **out);
int dgm_get_config(const dgm_config *c, dgm_config_view *out);
void dgm_free_config(dgm_config *c);

#ifdef __cplusplus
}
#endif
#endif /* DGMESH_H */
