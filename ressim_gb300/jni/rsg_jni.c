/*
 * JNI glue between a Java class no.uib.cipr.rs.gpu.RsgNative and the C ABI
 * of include/rsg.h: the C side a Java maintainer adds to RS to call the GPU
 * path.  Arrays are pinned with GetPrimitiveArrayCritical around each native
 * call, as the JNI glue MTJ ships does
 * (mtj/lib/jni/org_netlib_blas_NativeBLAS.c:44-52).  Handles travel to Java
 * as jlong.  Every function returns the rsg_status; the Java side maps 1..3
 * to IterativeSolverNotConvergedException and the others to SolverFailure,
 * as rs/src/no/uib/cipr/rs/numerics/LinearSolver.java:266-284 does.
 */
#include <jni.h>
#include <stdint.h>
#include <stdlib.h>

#include "rsg.h"

/* LinearSolver(RunSpec, Mesh, int[]): the pattern, copied to the device once */
JNIEXPORT jint JNICALL Java_no_uib_cipr_rs_gpu_RsgNative_csrCreate(JNIEnv* env, jclass cls, jlong ctx,
                                                                  jintArray rowptr, jintArray col, jlongArray out) {
  (void)cls;
  const jint n = (*env)->GetArrayLength(env, rowptr) - 1;
  const jint nnz = (*env)->GetArrayLength(env, col);
  rsg_csr* A = 0;
  jint* prp = (*env)->GetPrimitiveArrayCritical(env, rowptr, 0);
  jint* pcol = (*env)->GetPrimitiveArrayCritical(env, col, 0);
  rsg_status st = rsg_csr_create((rsg_ctx*)(intptr_t)ctx, n, nnz, (const int32_t*)prp, (const int32_t*)pcol, &A);
  (*env)->ReleasePrimitiveArrayCritical(env, col, pcol, JNI_ABORT);
  (*env)->ReleasePrimitiveArrayCritical(env, rowptr, prp, JNI_ABORT);
  jlong h = (jlong)(intptr_t)A;
  (*env)->SetLongArrayRegion(env, out, 0, 1, &h);
  return st;
}

/* CompRowMatrix.getData() after assembly */
JNIEXPORT jint JNICALL Java_no_uib_cipr_rs_gpu_RsgNative_csrSetValues(JNIEnv* env, jclass cls, jlong csr,
                                                                     jdoubleArray values) {
  (void)cls;
  double* pv = (*env)->GetPrimitiveArrayCritical(env, values, 0);
  rsg_status st = rsg_csr_set_values((rsg_csr*)(intptr_t)csr, pv);
  (*env)->ReleasePrimitiveArrayCritical(env, values, pv, JNI_ABORT);
  return st;
}

/* Preconditioner.setMatrix(A) */
JNIEXPORT jint JNICALL Java_no_uib_cipr_rs_gpu_RsgNative_setup(JNIEnv* env, jclass cls, jlong solver, jlong csr) {
  (void)env;
  (void)cls;
  return rsg_solver_setup((rsg_solver*)(intptr_t)solver, (rsg_csr*)(intptr_t)csr);
}

/* IterativeSolver.solve(A, b, x): x is the initial guess and is overwritten */
JNIEXPORT jint JNICALL Java_no_uib_cipr_rs_gpu_RsgNative_solve(JNIEnv* env, jclass cls, jlong solver, jlong csr,
                                                              jdoubleArray b, jdoubleArray x, jintArray iters,
                                                              jdoubleArray resid) {
  (void)cls;
  rsg_solve_info info;
  double* pb = (*env)->GetPrimitiveArrayCritical(env, b, 0);
  double* px = (*env)->GetPrimitiveArrayCritical(env, x, 0);
  rsg_status st = rsg_solver_solve((rsg_solver*)(intptr_t)solver, (rsg_csr*)(intptr_t)csr, pb, px, &info);
  (*env)->ReleasePrimitiveArrayCritical(env, x, px, 0);
  (*env)->ReleasePrimitiveArrayCritical(env, b, pb, JNI_ABORT);
  (*env)->SetIntArrayRegion(env, iters, 0, 1, &info.iterations);
  (*env)->SetDoubleArrayRegion(env, resid, 0, 1, &info.residual);
  return st;
}

/* Discretisation.solve(dt): one time step; newton[0] = pressure Newton iterations */
JNIEXPORT jint JNICALL Java_no_uib_cipr_rs_gpu_RsgNative_simStep(JNIEnv* env, jclass cls, jlong sim, jdouble dt,
                                                                jintArray newton) {
  (void)cls;
  rsg_step_info info;
  rsg_status st = rsg_sim_step((rsg_sim*)(intptr_t)sim, dt, &info);
  (*env)->SetIntArrayRegion(env, newton, 0, 1, &info.newton_iterations);
  return st;
}

/* Several fields stepped together (one persistent pressure-solver launch per
 * Newton iteration); sims: handles, dt: one step length per field; per field
 * newton[i] and statuses[i]. */
JNIEXPORT jint JNICALL Java_no_uib_cipr_rs_gpu_RsgNative_ensembleStepBatched(JNIEnv* env, jclass cls,
                                                                            jlongArray sims, jdoubleArray dt,
                                                                            jint precision, jintArray newton,
                                                                            jintArray statuses) {
  (void)cls;
  const jint count = (*env)->GetArrayLength(env, sims);
  if (count <= 0) return RSG_BAD_ARG;
  rsg_sim** hs = malloc(sizeof(rsg_sim*) * (size_t)count);
  rsg_step_info* infos = malloc(sizeof(rsg_step_info) * (size_t)count);
  int32_t* sts = malloc(sizeof(int32_t) * (size_t)count);
  rsg_status st = RSG_BAD_ARG;
  if (hs && infos && sts) {
    jlong* ph = (*env)->GetPrimitiveArrayCritical(env, sims, 0);
    for (jint i = 0; i < count; ++i) hs[i] = (rsg_sim*)(intptr_t)ph[i];
    (*env)->ReleasePrimitiveArrayCritical(env, sims, ph, JNI_ABORT);
    double* pdt = (*env)->GetPrimitiveArrayCritical(env, dt, 0);
    st = rsg_ensemble_step_batched(count, hs, pdt, precision, infos, sts);
    (*env)->ReleasePrimitiveArrayCritical(env, dt, pdt, JNI_ABORT);
    for (jint i = 0; i < count; ++i) {
      jint nt = infos[i].newton_iterations, s = sts[i];
      (*env)->SetIntArrayRegion(env, newton, i, 1, &nt);
      (*env)->SetIntArrayRegion(env, statuses, i, 1, &s);
    }
  }
  free(hs);
  free(infos);
  free(sts);
  return st;
}

/* L_MPFA.calculateTransmissibilities(mesh, K) in place of O_MPFA's */
JNIEXPORT jint JNICALL Java_no_uib_cipr_rs_gpu_RsgNative_meshComputeLmpfa(JNIEnv* env, jclass cls, jlong mesh) {
  (void)env;
  (void)cls;
  return rsg_mesh_compute_lmpfa((rsg_mesh*)(intptr_t)mesh);
}

/* new PressureDiscretisation(mesh, bc).getSolution(): bc as parallel arrays
 * of element indices and pressures; x receives the solution */
JNIEXPORT jint JNICALL Java_no_uib_cipr_rs_gpu_RsgNative_upscalePressure(JNIEnv* env, jclass cls, jlong mesh,
                                                                        jintArray cells, jdoubleArray values,
                                                                        jdoubleArray x, jintArray iters) {
  (void)cls;
  rsg_solve_info info;
  const jint nbc = (*env)->GetArrayLength(env, cells);
  jint* pc = (*env)->GetPrimitiveArrayCritical(env, cells, 0);
  double* pv = (*env)->GetPrimitiveArrayCritical(env, values, 0);
  double* px = (*env)->GetPrimitiveArrayCritical(env, x, 0);
  rsg_status st = rsg_upscale_pressure((rsg_mesh*)(intptr_t)mesh, nbc, (const int32_t*)pc, pv, px, &info);
  (*env)->ReleasePrimitiveArrayCritical(env, x, px, 0);
  (*env)->ReleasePrimitiveArrayCritical(env, values, pv, JNI_ABORT);
  (*env)->ReleasePrimitiveArrayCritical(env, cells, pc, JNI_ABORT);
  (*env)->SetIntArrayRegion(env, iters, 0, 1, &info.iterations);
  return st;
}

/* LocalFlowRateAverage.computeDarcyFlux: flux[c] = sum_k t_k p[k] per connection */
JNIEXPORT jint JNICALL Java_no_uib_cipr_rs_gpu_RsgNative_connectionFlux(JNIEnv* env, jclass cls, jlong mesh,
                                                                       jdoubleArray p, jdoubleArray flux) {
  (void)cls;
  double* pp = (*env)->GetPrimitiveArrayCritical(env, p, 0);
  double* pf = (*env)->GetPrimitiveArrayCritical(env, flux, 0);
  rsg_status st = rsg_mesh_connection_flux((rsg_mesh*)(intptr_t)mesh, pp, pf);
  (*env)->ReleasePrimitiveArrayCritical(env, flux, pf, 0);
  (*env)->ReleasePrimitiveArrayCritical(env, p, pp, JNI_ABORT);
  return st;
}
