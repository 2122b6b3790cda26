// pfm.cpp — the reference's HDR dump format (rendering/hdrimage.cpp:6-66):
// "PF\n", "<width> <height>\n", "-1.000000\n" (little-endian scale), then
// width*height RGB float triples, row 0 first (the bottom row, as GL reads
// images back). Host-only helpers for image diffs of drv_apply /
// drv_bruteforce_rsm output copied to the host.
#include <cstdio>
#include <cstring>

#include "../../include/drv.h"

extern "C" drv_status drv_write_pfm(const char* path, const float* rgb, int32_t width, int32_t height,
                                    int32_t channels) {
  if (!path || !rgb || width < 1 || height < 1 || (channels != 3 && channels != 4)) return DRV_ERR_INVALID_ARG;
  FILE* f = std::fopen(path, "wb");
  if (!f) return DRV_ERR_INVALID_ARG;
  bool ok = std::fprintf(f, "PF\n%d %d\n-1.000000\n", width, height) > 0;
  for (size_t i = 0; ok && i < (size_t)width * height; ++i)
    ok = std::fwrite(rgb + i * channels, sizeof(float), 3, f) == 3;
  ok = std::fclose(f) == 0 && ok;
  return ok ? DRV_OK : DRV_ERR_INVALID_ARG;
}

extern "C" drv_status drv_read_pfm(const char* path, float* rgb, int64_t capacity_pixels, int32_t* width,
                                   int32_t* height) {
  if (!path || !width || !height) return DRV_ERR_INVALID_ARG;
  FILE* f = std::fopen(path, "rb");
  if (!f) return DRV_ERR_INVALID_ARG;
  char magic[3] = {0, 0, 0};
  int w = 0, h = 0;
  char scale[32] = {0};
  drv_status st = DRV_OK;
  if (std::fread(magic, 1, 3, f) != 3 || std::memcmp(magic, "PF\n", 3) != 0 ||
      std::fscanf(f, "%d %d", &w, &h) != 2 || w < 1 || h < 1 || std::fscanf(f, "%31s", scale) != 1 ||
      std::fgetc(f) != '\n' || scale[0] != '-') {
    st = DRV_ERR_INVALID_ARG;  // not an RGB little-endian PFM
  } else {
    *width = w;
    *height = h;
    if (rgb) {
      if ((int64_t)w * h > capacity_pixels)
        st = DRV_ERR_CAPACITY;
      else if (std::fread(rgb, sizeof(float), (size_t)w * h * 3, f) != (size_t)w * h * 3)
        st = DRV_ERR_INVALID_ARG;
    }
  }
  std::fclose(f);
  return st;
}
