/* The C ABI from plain C (C99): the host-side entry points a C caller of
 * libesr_gb300.so uses before any device work -- the tutorial mesh, the
 * stable CSR of a Reducer index, reverse Cuthill-McKee and the tile
 * partition.  Writes each result as raw little-endian int64 to
 * <outdir>/<name>.bin for the Python test to compare.  Usage:
 *   c_abi_host <n> <max_part> <outdir> */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "esr_gb300.h"

static int dump(const char *dir, const char *name, const int64_t *a, int64_t count) {
  char path[4096];
  snprintf(path, sizeof path, "%s/%s.bin", dir, name);
  FILE *f = fopen(path, "wb");
  if (!f) return 1;
  size_t w = fwrite(a, sizeof(int64_t), (size_t)count, f);
  fclose(f);
  return w != (size_t)count;
}

#define CHECK(call)                                                    \
  do {                                                                 \
    if ((call) != ESR_OK) {                                            \
      fprintf(stderr, "%s failed: %s\n", #call, esr_last_error());     \
      return 1;                                                        \
    }                                                                  \
  } while (0)

int main(int argc, char **argv) {
  if (argc != 4) return 2;
  const int64_t n = atoll(argv[1]), max_part = atoll(argv[2]);
  const char *dir = argv[3];
  if (esr_abi_version() != ESR_GB300_ABI_VERSION) {
    fprintf(stderr, "ABI version %d, header %d\n", esr_abi_version(), ESR_GB300_ABI_VERSION);
    return 1;
  }
  int64_t nc, ne, nbc, np;
  CHECK(esr_mesh_sizes(n, &nc, &ne, &nbc, &np));
  int64_t *src = malloc(ne * sizeof *src), *dst = malloc(ne * sizeof *dst);
  int64_t *cells = malloc(3 * nc * sizeof *cells), *bcells = malloc(nbc * sizeof *bcells);
  int64_t *bpoints = malloc(2 * nbc * sizeof *bpoints);
  double *points = malloc(2 * np * sizeof *points);
  int64_t *rowptr = malloc((nc + 1) * sizeof *rowptr), *perm = malloc(ne * sizeof *perm);
  int64_t *order = malloc(nc * sizeof *order), *part = malloc(nc * sizeof *part);
  if (!src || !dst || !cells || !bcells || !bpoints || !points || !rowptr || !perm || !order || !part) return 1;
  CHECK(esr_mesh_triangular(n, src, dst, cells, bcells, bpoints, points));
  CHECK(esr_csr_from_index(dst, ne, nc, rowptr, perm));
  CHECK(esr_rcm_order(nc, ne, src, dst, order));
  int64_t nparts = 0;
  CHECK(esr_bisect_partition(nc, ne, src, dst, max_part, part, &nparts));
  int64_t sizes[5] = {nc, ne, nbc, np, nparts};
  int bad = dump(dir, "sizes", sizes, 5) || dump(dir, "src", src, ne) || dump(dir, "rowptr", rowptr, nc + 1) ||
            dump(dir, "perm", perm, ne) || dump(dir, "order", order, nc) || dump(dir, "part", part, nc);
  /* an out-of-range index is an error with a message, not a crash */
  dst[0] = nc;
  if (esr_csr_from_index(dst, ne, nc, rowptr, perm) != ESR_ERR_ARG || strlen(esr_last_error()) == 0) bad = 1;
  free(src); free(dst); free(cells); free(bcells); free(bpoints); free(points);
  free(rowptr); free(perm); free(order); free(part);
  return bad;
}
