/*
 * capi_fuse_client.c -- a plain C99 host program that fuses depth frames and meshes the volume through the C ABI
 * of include/voxelhash_gb300.h only: vh_create -> vh_integrate (host depth) per frame -> vh_extract_mesh ->
 * vh_copy_mesh -> vh_destroy.  Built and run by tests/test_gpu_c_client.py, which compares its output with the
 * Python path and with the oracle.
 *
 * usage: capi_fuse_client <frames.bin> <out.bin>
 *   frames.bin: int32 width, height, frame count; float fx, fy, cx, cy, voxel size, truncation; uint32 hash
 *               buckets, max blocks; then per frame 12 floats (R row-major, t) and width*height float depths.
 *   out.bin:    uint64 block count, observed voxels, triangle count; then 9 floats per triangle.
 */
#include <stdio.h>
#include <stdlib.h>

#include "voxelhash_gb300.h"

static int read_exact(FILE* f, void* dst, size_t bytes) { return fread(dst, 1, bytes, f) == bytes; }

static int fail(const char* what, vh_status s, const vh_volume* v) {
  fprintf(stderr, "%s: %s (%s)\n", what, vh_status_string(s), v ? vh_last_error(v) : "");
  return 1;
}

int main(int argc, char** argv) {
  int32_t hdr[3];
  float fk[6];
  uint32_t sizes[2];
  FILE* in;
  FILE* out;
  vh_params params;
  vh_intrinsics K;
  vh_volume* vol = NULL;
  float* depth = NULL;
  float* soup = NULL;
  size_t npx, ntri = 0;
  uint64_t blocks = 0, observed = 0, header[3];
  int32_t f;
  vh_status s;
  int rc = 1;

  if (argc != 3) {
    fprintf(stderr, "usage: %s <frames.bin> <out.bin>\n", argv[0]);
    return 2;
  }
  in = fopen(argv[1], "rb");
  if (!in) return fail("open input", VH_ERR_IO, NULL);
  if (!read_exact(in, hdr, sizeof hdr) || !read_exact(in, fk, sizeof fk) || !read_exact(in, sizes, sizeof sizes)) {
    fclose(in);
    return fail("read header", VH_ERR_IO, NULL);
  }
  K.width = hdr[0];
  K.height = hdr[1];
  K.fx = fk[0];
  K.fy = fk[1];
  K.cx = fk[2];
  K.cy = fk[3];
  vh_params_default(&params);
  params.voxel_size = fk[4];
  params.truncation_distance = fk[5];
  params.hash_buckets = sizes[0];
  params.max_blocks = sizes[1];
  s = vh_create(&params, NULL, &vol);
  if (s != VH_OK) {
    fclose(in);
    return fail("vh_create", s, NULL);
  }
  npx = (size_t)K.width * (size_t)K.height;
  depth = (float*)malloc(npx * sizeof(float));
  if (!depth) goto done;
  for (f = 0; f < hdr[2]; ++f) {
    vh_pose T;
    if (!read_exact(in, T.R, sizeof T.R) || !read_exact(in, T.t, sizeof T.t) ||
        !read_exact(in, depth, npx * sizeof(float))) {
      fail("read frame", VH_ERR_IO, NULL);
      goto done;
    }
    s = vh_integrate(vol, depth, 0, &K, &T, 1, NULL);
    if (s == VH_OK) s = vh_synchronize(vol, NULL);
    if (s != VH_OK) {
      fail("vh_integrate", s, vol);
      goto done;
    }
  }
  s = vh_extract_mesh(vol, 0.0f, &ntri, NULL);
  if (s != VH_OK) {
    fail("vh_extract_mesh", s, vol);
    goto done;
  }
  soup = (float*)malloc((ntri ? ntri : 1) * 9 * sizeof(float));
  if (!soup) goto done;
  s = vh_copy_mesh(vol, soup, ntri, 0, NULL);
  if (s == VH_OK) s = vh_block_count(vol, &blocks);
  if (s == VH_OK) s = vh_observed_voxel_count(vol, &observed);
  if (s != VH_OK) {
    fail("read results", s, vol);
    goto done;
  }
  out = fopen(argv[2], "wb");
  if (!out) {
    fail("open output", VH_ERR_IO, NULL);
    goto done;
  }
  header[0] = blocks;
  header[1] = observed;
  header[2] = (uint64_t)ntri;
  if (fwrite(header, sizeof header, 1, out) == 1 && (ntri == 0 || fwrite(soup, 9 * sizeof(float), ntri, out) == ntri)) {
    rc = 0;
  }
  fclose(out);
done:
  free(soup);
  free(depth);
  fclose(in);
  vh_destroy(vol);
  return rc;
}
