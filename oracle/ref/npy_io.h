/*
  .npy reading and writing for the reference-driving programs under
  oracle/ref (golden_gen.cpp, cpu_ref_bench.cpp).  Test infrastructure only.
*/
#pragma once
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <string>
#include <vector>

static void write_npy(const std::string &path, const char *descr,
                      const void *data, size_t elsize, const std::vector<long> &shape) {
  FILE *fp = fopen(path.c_str(), "wb");
  if (!fp) {
    fprintf(stderr, "cannot write %s\n", path.c_str());
    exit(1);
  }
  std::string shp = "(";
  size_t n = 1;
  for (size_t i = 0; i < shape.size(); i++) {
    shp += std::to_string(shape[i]);
    shp += (shape.size() == 1) ? "," : (i + 1 < shape.size() ? ", " : "");
    n *= (size_t)shape[i];
  }
  shp += ")";
  std::string hdr = std::string("{'descr': '") + descr +
                    "', 'fortran_order': False, 'shape': " + shp + ", }";
  size_t total = 10 + hdr.size() + 1;
  size_t pad = (64 - total % 64) % 64;
  hdr += std::string(pad, ' ');
  hdr += "\n";
  unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
  fwrite(magic, 1, 8, fp);
  uint16_t hl = (uint16_t)hdr.size();
  fwrite(&hl, 2, 1, fp);
  fwrite(hdr.data(), 1, hdr.size(), fp);
  fwrite(data, elsize, n, fp);
  fclose(fp);
}

/* Minimal reader for the little-endian C-order arrays the fixture script
   writes ('<f8' or '<i4'). */
template <typename T>
static std::vector<T> read_npy(const std::string &path, std::vector<long> *shape_out = NULL) {
  FILE *fp = fopen(path.c_str(), "rb");
  if (!fp) {
    fprintf(stderr, "cannot read %s\n", path.c_str());
    exit(1);
  }
  unsigned char magic[8];
  if (fread(magic, 1, 8, fp) != 8) exit(1);
  uint16_t hl = 0;
  if (fread(&hl, 2, 1, fp) != 1) exit(1);
  std::string hdr(hl, ' ');
  if (fread(&hdr[0], 1, hl, fp) != hl) exit(1);
  size_t p = hdr.find("'shape': (");
  std::vector<long> shape;
  if (p != std::string::npos) {
    p += 10;
    while (hdr[p] != ')') {
      if (hdr[p] >= '0' && hdr[p] <= '9') {
        long v = 0;
        while (hdr[p] >= '0' && hdr[p] <= '9') v = 10 * v + (hdr[p++] - '0');
        shape.push_back(v);
      } else {
        p++;
      }
    }
  }
  size_t n = 1;
  for (long s : shape) n *= (size_t)s;
  std::vector<T> out(n);
  if (n && fread(out.data(), sizeof(T), n, fp) != n) exit(1);
  fclose(fp);
  if (shape_out) *shape_out = shape;
  return out;
}

