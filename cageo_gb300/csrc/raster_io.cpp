// raster_io.cpp -- A10 raster I/O in the reference's file formats.
//
// Header (src/utils/utils.cpp:58-112): whitespace-separated tag/value
// pairs; tags ncols nrows xllcorner yllcorner cellsize NODATA_value
// byteorder|BYTEORDER (MSBFIRST|LSBFIRST).  An unknown tag or byte order is
// an error (the reference exits).  Rasters (src/utils/SystemUtils.h:53-86):
// raw native-endian float32 row-major; the reference reads the whole file
// into the buffer without a size check, here a size mismatch is an error.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include "cageo.h"
#include "guard.h"

static cageo_status read_header(const char* path, cageo_raster_info* info) {
  if (!path || !info) {
    cageo::set_error("invalid argument: null header path or output");
    return CAGEO_ERR_ARGUMENT;
  }
  std::ifstream f(path);
  if (!f.is_open()) {
    cageo::set_error("unable to open header \"%s\"", path);
    return CAGEO_ERR_IO;
  }
  cageo_raster_info r{};
  r.nodata_value = 0.0f;
  bool have_cols = false, have_rows = false;
  std::string tag;
  while (f >> tag) {
    if (tag == "ncols") { f >> r.ncols; have_cols = true; }
    else if (tag == "nrows") { f >> r.nrows; have_rows = true; }
    else if (tag == "xllcorner") f >> r.xllcorner;
    else if (tag == "yllcorner") f >> r.yllcorner;
    else if (tag == "cellsize") f >> r.cellsize;
    else if (tag == "NODATA_value") f >> r.nodata_value;
    else if (tag == "byteorder" || tag == "BYTEORDER") {
      std::string v;
      f >> v;
      if (v == "MSBFIRST") r.byteorder_msb = 1;
      else if (v == "LSBFIRST") r.byteorder_msb = 0;
      else {
        cageo::set_error("unrecognized byte order value: %s", v.c_str());
        return CAGEO_ERR_FORMAT;
      }
    } else {
      cageo::set_error("unrecognized tag value: %s", tag.c_str());
      return CAGEO_ERR_FORMAT;
    }
    if (f.fail()) {
      cageo::set_error("bad value for tag %s in \"%s\"", tag.c_str(), path);
      return CAGEO_ERR_FORMAT;
    }
  }
  if (!have_cols || !have_rows || r.ncols <= 0 || r.nrows <= 0) {
    cageo::set_error("header \"%s\" lacks positive ncols/nrows", path);
    return CAGEO_ERR_FORMAT;
  }
  *info = r;
  return CAGEO_OK;
}

extern "C" cageo_status cageo_read_header(const char* path, cageo_raster_info* info) {
  return cageo::guarded("cageo_read_header", [&] { return read_header(path, info); });
}

extern "C" cageo_status cageo_write_header(const char* path, const cageo_raster_info* info) {
  if (!path || !info) {
    cageo::set_error("invalid argument: null header path or input");
    return CAGEO_ERR_ARGUMENT;
  }
  FILE* f = std::fopen(path, "w");
  if (!f) {
    cageo::set_error("unable to open \"%s\" for writing", path);
    return CAGEO_ERR_IO;
  }
  const int put =
      std::fprintf(f, "ncols         %d\nnrows         %d\nxllcorner     %.10g\nyllcorner     %.10g\n"
                      "cellsize      %.9g\nNODATA_value  %.9g\nbyteorder     %s\n",
                   info->ncols, info->nrows, info->xllcorner, info->yllcorner, info->cellsize,
                   info->nodata_value, info->byteorder_msb ? "MSBFIRST" : "LSBFIRST");
  if ((std::fclose(f) != 0) || put < 0) {
    cageo::set_error("short write to \"%s\"", path);
    return CAGEO_ERR_IO;
  }
  return CAGEO_OK;
}

extern "C" cageo_status cageo_read_raster(const char* path, float* h_out, size_t count) {
  if (!path || !h_out) {
    cageo::set_error("invalid argument: null raster path or output");
    return CAGEO_ERR_ARGUMENT;
  }
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    cageo::set_error("unable to open file \"%s\"", path);
    return CAGEO_ERR_IO;
  }
  std::fseek(f, 0, SEEK_END);
  long long size = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (size != (long long)(count * sizeof(float))) {
    std::fclose(f);
    cageo::set_error("\"%s\" holds %lld bytes, expected %zu", path, size, count * sizeof(float));
    return CAGEO_ERR_FORMAT;
  }
  size_t got = std::fread(h_out, sizeof(float), count, f);
  std::fclose(f);
  if (got != count) {
    cageo::set_error("short read from \"%s\"", path);
    return CAGEO_ERR_IO;
  }
  return CAGEO_OK;
}

extern "C" cageo_status cageo_write_raster(const char* path, const float* h_data, size_t count) {
  if (!path || !h_data) {
    cageo::set_error("invalid argument: null raster path or input");
    return CAGEO_ERR_ARGUMENT;
  }
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    cageo::set_error("unable to open \"%s\" for writing", path);
    return CAGEO_ERR_IO;
  }
  const size_t put = std::fwrite(h_data, sizeof(float), count, f);
  const bool closed = std::fclose(f) == 0;
  if (put != count || !closed) {
    cageo::set_error("short write to \"%s\"", path);
    return CAGEO_ERR_IO;
  }
  return CAGEO_OK;
}
