/* A plain C caller of the library: reads a line list and one layer from
 * binary files, runs create -> od_size -> od -> od_stats -> destroy through
 * include/clblm_gb300.h, and writes the optical depth.  Used by
 * tests/test_cabi_c.py (no Python, torch or ctypes on this path).
 *
 *   od_call <lines.bin> <layer.bin> <out.bin> <precision>
 *
 * lines.bin: int64 n, then vnu[n] f64, sp, alfa, epp f32, mol i32,
 *            hwhm, tmpalf, pshift f32, iflg i32
 * layer.bin: int32 nmol, int32 mol_id[nmol], f64 w[nmol], f64 wtot, pave,
 *            tave, v1, v2, dv_normal, dv_narrow
 * out.bin:   int64 nsamp, f64 dv, int64 nlin, lincnt, nshrunk, npanels,
 *            then f64 od[nsamp]
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "clblm_gb300.h"

static void* read_n(FILE* f, size_t each, int64_t n) {
  void* p = malloc(each * (size_t)(n > 0 ? n : 1));
  if (!p || fread(p, each, (size_t)n, f) != (size_t)n) {
    fprintf(stderr, "short read\n");
    exit(2);
  }
  return p;
}

int main(int argc, char** argv) {
  if (argc != 5) {
    fprintf(stderr, "usage: od_call lines.bin layer.bin out.bin precision\n");
    return 2;
  }
  FILE* fl = fopen(argv[1], "rb");
  FILE* fy = fopen(argv[2], "rb");
  if (!fl || !fy) return 2;
  clblm_lines_t L;
  memset(&L, 0, sizeof L);
  if (fread(&L.n, 8, 1, fl) != 1) return 2;
  L.vnu = read_n(fl, 8, L.n);
  L.sp = read_n(fl, 4, L.n);
  L.alfa = read_n(fl, 4, L.n);
  L.epp = read_n(fl, 4, L.n);
  L.mol = read_n(fl, 4, L.n);
  L.hwhm = read_n(fl, 4, L.n);
  L.tmpalf = read_n(fl, 4, L.n);
  L.pshift = read_n(fl, 4, L.n);
  L.iflg = read_n(fl, 4, L.n);
  fclose(fl);

  int32_t nmol = 0;
  if (fread(&nmol, 4, 1, fy) != 1) return 2;
  int32_t* ids = read_n(fy, 4, nmol);
  double* w = read_n(fy, 8, nmol);
  double sc[7];
  if (fread(sc, 8, 7, fy) != 7) return 2;
  fclose(fy);

  clblm_layer_t lay = {nmol, ids, w, sc[0], sc[1], sc[2], 0.0, 0.0, 1};
  clblm_grid_t grid = {sc[3], sc[4], sc[5], sc[6], 0.0, 4.0, 0.04};
  clblm_od_ctrl_t ctrl;
  memset(&ctrl, 0, sizeof ctrl);
  ctrl.jrad = 1;
  ctrl.line_rejec = 1;
  ctrl.xself = ctrl.xfrgn = 1.0;
  ctrl.contnm_off = 1;
  ctrl.precision = atoi(argv[4]);

  clblm_handle_t* h = NULL;
  int rc = clblm_gpu_create(&L, NULL, 0, &h);
  if (rc != CLBLM_OK) {
    fprintf(stderr, "create: %d %s\n", rc, clblm_gpu_last_error(NULL));
    return 1;
  }
  int64_t nsamp = 0;
  double dv = 0.0;
  rc = clblm_gpu_od_size(h, &lay, &grid, &ctrl, &nsamp, &dv);
  if (rc != CLBLM_OK) {
    fprintf(stderr, "od_size: %d %s\n", rc, clblm_gpu_last_error(h));
    return 1;
  }
  double* od = malloc(sizeof(double) * (size_t)nsamp);
  rc = clblm_gpu_od(h, &lay, &grid, &ctrl, od, nsamp, CLBLM_OUT_HOST);
  if (rc != CLBLM_OK) {
    fprintf(stderr, "od: %d %s\n", rc, clblm_gpu_last_error(h));
    return 1;
  }
  clblm_od_stats_t st;
  rc = clblm_gpu_od_stats(h, &st);
  if (rc != CLBLM_OK) return 1;
  /* a too-small buffer is refused with CLBLM_ERR_CAPACITY */
  if (clblm_gpu_od(h, &lay, &grid, &ctrl, od, nsamp - 1, CLBLM_OUT_HOST) != CLBLM_ERR_CAPACITY) {
    fprintf(stderr, "capacity not checked\n");
    return 1;
  }
  clblm_gpu_destroy(h);

  FILE* fo = fopen(argv[3], "wb");
  if (!fo) return 2;
  int64_t cnt[4] = {st.nlin, st.lincnt, st.nshrunk, st.npanels};
  fwrite(&nsamp, 8, 1, fo);
  fwrite(&dv, 8, 1, fo);
  fwrite(cnt, 8, 4, fo);
  fwrite(od, 8, (size_t)nsamp, fo);
  fclose(fo);
  printf("od_call: %lld points, dv %.6g\n", (long long)nsamp, dv);
  return 0;
}
