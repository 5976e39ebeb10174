/* A plain C client of the library's C ABI (include/tcw_b200.h): creates a
 * handle, computes one map from host buffers, then the same atoms as a
 * two-template batched plan (blocking and pipelined from page-locked
 * buffers), and prints the result records as JSON; without a device it
 * prints the status and message instead.  Built by tests/test_c_abi.py with
 * gcc against the shared library. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "tcw_b200.h"

int main(int argc, char **argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s atoms.bin window\n", argv[0]);
    return 2;
  }
  /* atoms.bin: u32 numAtoms, TAtom, t0_data, N_t0, N_tau, then t0s, taus
   * (u32) and the (numAtoms, 7) float32 atoms */
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  uint32_t hdr[5];
  if (fread(hdr, sizeof(uint32_t), 5, f) != 5) return 2;
  const uint32_t numAtoms = hdr[0], TAtom = hdr[1], t0_data = hdr[2], N_t0 = hdr[3], N_tau = hdr[4];
  uint32_t *t0s = malloc(sizeof(uint32_t) * N_t0), *taus = malloc(sizeof(uint32_t) * N_tau);
  float *atoms = malloc(sizeof(float) * 7u * numAtoms);
  float *F = malloc(sizeof(float) * (size_t)N_t0 * N_tau);
  if (fread(t0s, sizeof(uint32_t), N_t0, f) != N_t0 || fread(taus, sizeof(uint32_t), N_tau, f) != N_tau ||
      fread(atoms, sizeof(float), 7u * numAtoms, f) != 7u * numAtoms)
    return 2;
  fclose(f);
  printf("{\"abi\": %d, ", tcw_abi_version());
  tcw_handle *h = NULL;
  int rc = tcw_create(&h, 0);
  if (rc != TCW_OK) {
    printf("\"create\": %d, \"error\": \"%s\"}\n", rc, tcw_strerror(rc));
    return 0;
  }
  tcw_result r;
  rc = tcw_map_plain_host(h, atoms, numAtoms, TAtom, t0_data, atoi(argv[2]), t0s, N_t0, taus, N_tau,
                          F, &r, TCW_FLAG_LNBTSG | TCW_FLAG_POSTERIORS);
  if (rc != TCW_OK) {
    printf("\"map\": %d, \"error\": \"%s\"}\n", rc, tcw_last_error(h));
    tcw_destroy(h);
    return 0;
  }
  printf("\"map\": 0, \"maxF\": %.9g, \"argmax\": %lld, \"lnBtSG\": %.17g, \"t0_mp_idx\": %lld, "
         "\"tau_mp_idx\": %lld, \"F00\": %.9g, ",
         r.maxF, (long long)r.argmax, r.lnBtSG, (long long)r.t0_mp_idx, (long long)r.tau_mp_idx,
         F[0]);
  /* the same atoms and grids as a batched plan of two templates (rect, exp),
   * run blocking, then twice pipelined from page-locked buffers */
  tcw_template_desc desc[2];
  for (int k = 0; k < 2; k++) {
    desc[k].atom_offset = 0;
    desc[k].t0_offset = 0;
    desc[k].tau_offset = 0;
    desc[k].numAtoms = numAtoms;
    desc[k].TAtom = TAtom;
    desc[k].t0_data = t0_data;
    desc[k].window = k == 0 ? TCW_WINDOW_RECT : TCW_WINDOW_EXP;
    desc[k].N_t0 = N_t0;
    desc[k].N_tau = N_tau;
  }
  tcw_plan *plan = NULL;
  rc = tcw_plan_create(h, desc, 2, t0s, N_t0, taus, N_tau, NULL, TCW_FLAG_LNBTSG, &plan);
  tcw_result pr[2];
  if (rc == TCW_OK) rc = tcw_plan_run_host(h, plan, atoms, pr);
  float *patoms = NULL;
  tcw_result *pres = NULL;
  if (rc == TCW_OK) rc = tcw_pinned_alloc((void **)&patoms, sizeof(float) * 7u * numAtoms);
  if (rc == TCW_OK) rc = tcw_pinned_alloc((void **)&pres, sizeof(tcw_result) * 4);
  if (rc == TCW_OK) {
    for (uint32_t i = 0; i < 7u * numAtoms; i++) patoms[i] = atoms[i];
    rc = tcw_plan_run_host_async(h, plan, patoms, pres);
    if (rc == TCW_OK) rc = tcw_plan_run_host_async(h, plan, patoms, pres + 2);
    if (rc == TCW_OK) rc = tcw_sync(h, 60000);
  }
  if (rc != TCW_OK) {
    printf("\"plan\": %d, \"error\": \"%s\"}\n", rc, tcw_last_error(h));
  } else {
    int same = 1;
    for (int k = 0; k < 4; k++)
      same = same && pres[k].maxF == pr[k % 2].maxF && pres[k].argmax == pr[k % 2].argmax &&
             pres[k].lnBtSG == pr[k % 2].lnBtSG;
    printf("\"plan\": 0, \"plan_maxF\": [%.9g, %.9g], \"plan_argmax\": [%lld, %lld], "
           "\"pipelined_equal\": %s}\n",
           pr[0].maxF, pr[1].maxF, (long long)pr[0].argmax, (long long)pr[1].argmax,
           same ? "true" : "false");
  }
  tcw_pinned_free(patoms);
  tcw_pinned_free(pres);
  if (plan) tcw_plan_destroy(plan);
  tcw_destroy(h);
  free(t0s);
  free(taus);
  free(atoms);
  free(F);
  return 0;
}
