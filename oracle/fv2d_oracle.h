/*
 * fv2d oracle C interface -- TEST INFRASTRUCTURE ONLY.
 *
 * Two CPU libraries implement this interface:
 *   - the oracle port  (oracle/fv2d_oracle.cpp, symbols prefixed fvo_): a line-by-line CPU
 *     restatement of the reference solver step with variable-length cell face lists;
 *   - the reference harness (oracle/ref_harness.cpp, symbols prefixed fvr_): the reference's
 *     own, unmodified solver sources driven stage by stage.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load them, as the checker.
 * The product library never links or calls either one.
 *
 * Field ids for *_get(): every double array is returned in the reference's own (file) numbering.
 * Conservative/gradient blocks are SoA: p1 block, p2 block, p3 block, p4 block.
 */
#ifndef FV2D_ORACLE_H
#define FV2D_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum fvo_field {
    FVO_QBAR = 0,        /* 4N  Qbar conservative                                  */
    FVO_QSTAR = 1,       /* 4N  Q* (stage-driver output of stages 1 and 2)         */
    FVO_RES = 2,         /* 4N  residual of the last res() call                    */
    FVO_DT = 3,          /* N   time step of the current iteration                 */
    FVO_QBAR_GRAD = 4,   /* 8N  Qbar Qx p1..p4, Qy p1..p4                          */
    FVO_QSTAR_GRAD = 5,  /* 8N  Q* gradients                                       */
    FVO_QF1 = 6,         /* 4F  Qface_c1 p1..p4                                    */
    FVO_QF2 = 7,         /* 4F  Qface_c2 p1..p4                                    */
    FVO_VNC = 8,         /* 2F  Vn_avg, c_avg                                      */
    FVO_QBAR_PRIM = 9,   /* 4N  Qbar rho, u, v, P                                  */
    /* geometry (mesh) */
    FVO_G_AREA = 20, FVO_G_NX, FVO_G_NY, FVO_G_FCX, FVO_G_FCY,
    FVO_G_C1DX, FVO_G_C1DY, FVO_G_C2DX, FVO_G_C2DY, FVO_G_DXJ, FVO_G_DYJ,
    FVO_G_DIST, FVO_G_LX, FVO_G_LY, FVO_G_MX, FVO_G_MY,          /* per face (F) */
    FVO_G_VOL = 40, FVO_G_CCX, FVO_G_CCY, FVO_G_IXX, FVO_G_IYY, FVO_G_IXY, FVO_G_DELTA, /* per cell (N) */
    FVO_G_BCCX = 50, FVO_G_BCCY                                   /* per boundary face */
};

enum fvo_ifield {
    FVO_I_FC1 = 0,       /* F   face_cell1 (0-based)                              */
    FVO_I_FC2 = 1,       /* F   face_cell2 (0-based, or negative BC code)         */
    FVO_I_FP1 = 2,       /* F   face_point1                                       */
    FVO_I_FP2 = 3,       /* F   face_point2                                       */
    FVO_I_CFC = 4,       /* N   cell_face_count                                   */
    FVO_I_BCF = 5        /* Nb  BC_faces                                          */
};

/* sizes[]: num_points, num_faces, num_cells, numBC1, numBC2, numWALL, num_of_BC, stage */

/* case description for fvo_open_arrays (the fields of input.in after read_inputs) */
typedef struct fvo_case {
    int order;          /* solution_poly_order + 1                      */
    int eqn;            /* 1 EULER, 2 NS                                */
    int flux_solver;    /* 1 RUSANOV                                    */
    int limiter;        /* 0 NONE, 1 MINMOD, 2 SQUEEZE                  */
    int time_type;      /* 1 GLOBAL, 2 LOCAL                            */
    int time_scheme;    /* 2 SSP_RK3                                    */
    int bc1, bc2;       /* -1 FREESTREAM, -2 SLIP, -3 EXTRAP, -4 NO_SLIP */
    double cfl, gamma, R, mu, Pr, P, rho, u, v;
} fvo_case;

/* oracle port */
void*  fvo_open(const char* input_file);
void*  fvo_open_arrays(const fvo_case* cs, int np, int nf, int nc,
                       const double* x, const double* y,
                       const int* file_fp1, const int* file_fp2,
                       const int* file_fc1, const int* file_fc2);
void   fvo_close(void* h);
void   fvo_sizes(void* h, int* out8);
void   fvo_stage(void* h);
void   fvo_iterate(void* h, int n);
int    fvo_get(void* h, int field, double* out);
int    fvo_get_int(void* h, int field, int* out);
void   fvo_set_state(void* h, const double* q4n);
double fvo_time_iterations(void* h, int n);

/* reference harness */
void*  fvr_open(const char* input_file);
void   fvr_close(void* h);
void   fvr_sizes(void* h, int* out8);
void   fvr_stage(void* h);
void   fvr_iterate(void* h, int n);
int    fvr_get(void* h, int field, double* out);
int    fvr_get_int(void* h, int field, int* out);
void   fvr_set_state(void* h, const double* q4n);
double fvr_time_iterations(void* h, int n);

#ifdef __cplusplus
}
#endif
#endif
