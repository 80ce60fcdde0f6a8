/*
 * eporacle.h -- CPU FP64 restatement of ElastoPlasm's explicit MPM step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker for the GPU library
 * (include/epgpu.h): only the tests, the smoke check and the CPU baseline of
 * the benchmark load it.  The product never links or calls it.
 *
 * It follows the reference's kernels one by one, serially, in point order,
 * with the reference's array layout (column-major Julia arrays), scatter
 * order and sparse nonlocal bookkeeping; see eporacle.cpp for the file:line
 * each routine restates.  Parity status: the reference (Julia) cannot run in
 * this build environment, so the oracle is pinned by the reference's own
 * known-answer test (the elastic column collapse of test/testset/test_collapse.jl)
 * and by the closed-form and property checks in tests/, not by vectors
 * produced by the reference itself.
 */
#ifndef EPORACLE_H
#define EPORACLE_H

#include "../include/epgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct eporacle eporacle;

eporacle* eporacle_create(const ep_cfg* cfg, const ep_cmpr* cmpr, const ep_mesh_view* mesh, int64_t nmp);
int eporacle_upload(eporacle* o, const ep_mpts_view* m);
/* one cycle with the caller's dt and g; returns 0 or an ep_status */
int eporacle_step(eporacle* o, int32_t phase, double dt, const double* g, double* vmax_out);
/* the reference's inner loop for one checkpoint window (see epgpu_run) */
int eporacle_run(eporacle* o, int32_t phase, double T, double tg, double* t_inout, int64_t* nsteps_out);
int eporacle_download(eporacle* o, ep_mpts_view* m);
int eporacle_download_mesh(eporacle* o, ep_mesh_fields* f);
/* the element-to-node table as the reference builds it (e2n.jl:20-78), nn x nel, 1-based */
int eporacle_e2n(eporacle* o, int64_t* out);
/* worker threads for the point-parallel loops (1 = serial, exact reference order) */
void eporacle_set_threads(eporacle* o, int threads);
const char* eporacle_last_error(eporacle* o);
void eporacle_destroy(eporacle* o);

#ifdef __cplusplus
}
#endif

#endif
