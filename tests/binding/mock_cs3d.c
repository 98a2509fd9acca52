/* mock_cs3d.c -- TEST DOUBLE of the C ABI (include/cs3d.h) for the host
 * binding test: every entry point the binding calls prints one line
 * "CALL <name> <args>" and returns CS3D_OK, so that a CPU test can check the
 * call sequence that the reference's own RK loops issue through
 * cs3d_ref_binding.hpp.  Computes nothing. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cs3d.h"

struct cs3d_handle { int npts; int step; };
struct cs3d_op { int npts; };

const char *cs3d_last_error(void) { return "mock"; }
int cs3d_create(const cs3d_config *c, cs3d_handle **out) {
    cs3d_handle *h = (cs3d_handle *)calloc(1, sizeof(cs3d_handle));
    h->npts = c->Nx * c->Ny * c->Nz;
    printf("CALL create %d %d %d rk %d filter_step %d\n", c->Nx, c->Ny, c->Nz, c->rk, c->filter_step);
    *out = h;
    return CS3D_OK;
}
int cs3d_destroy(cs3d_handle *h) { printf("CALL destroy\n"); free(h); return CS3D_OK; }
int cs3d_set_initial_conditions(cs3d_handle *h, const double *r, const double *p, const double *u,
                                const double *v, const double *w) {
    (void)h; printf("CALL set_initial_conditions %.6f %.6f\n", r[0], u[1]); (void)p; (void)v; (void)w;
    return CS3D_OK;
}
int cs3d_pre_step(cs3d_handle *h) { h->step++; printf("CALL pre_step\n"); return CS3D_OK; }
int cs3d_sub_step(cs3d_handle *h, int s, int last) { (void)h; printf("CALL sub_step %d %d\n", s, last); return CS3D_OK; }
int cs3d_post_step(cs3d_handle *h) { (void)h; printf("CALL post_step\n"); return CS3D_OK; }
int cs3d_get_field(cs3d_handle *h, int f, double *out) {
    for (int i = 0; i < h->npts; i++) out[i] = f % 5 == 0 ? 1.0 : 0.0;
    if (f == 0) printf("CALL get_field 0..14\n");
    return CS3D_OK;
}
int cs3d_set_field(cs3d_handle *h, int f, const double *in) { (void)h; (void)in; printf("CALL set_field %d\n", f); return CS3D_OK; }
int cs3d_get_scalars(cs3d_handle *h, double *dt, double *time, int *ts) {
    if (dt) *dt = 1e-3;
    if (time) *time = 1e-3 * (h->step > 0 ? h->step - 1 : 0);
    if (ts) *ts = h->step;
    return CS3D_OK;
}
int cs3d_dump_solution(cs3d_handle *h, const char *prefix) { (void)h; printf("CALL dump_solution '%s'\n", prefix); return CS3D_OK; }
int cs3d_op_create(const cs3d_config *c, int dir, cs3d_op **out) {
    cs3d_op *o = (cs3d_op *)calloc(1, sizeof(cs3d_op));
    o->npts = c->Nx * c->Ny * c->Nz;
    printf("CALL op_create dir %d bc %d\n", dir, c->bc_type[dir]);
    *out = o;
    return CS3D_OK;
}
int cs3d_op_destroy(cs3d_op *o) { printf("CALL op_destroy\n"); free(o); return CS3D_OK; }
int cs3d_op_apply(cs3d_op *o, int kind, const double *in, double *out) { (void)o; (void)in; (void)out; printf("CALL op_apply %d\n", kind); return CS3D_OK; }
int cs3d_op_apply_host(cs3d_op *o, int kind, const double *in, double *out) {
    memcpy(out, in, sizeof(double) * (size_t)o->npts);
    printf("CALL op_apply_host %d\n", kind);
    return CS3D_OK;
}
int cs3d_op_get_stream(cs3d_op *o, void **s) { (void)o; *s = NULL; return CS3D_OK; }
