// drainage_main.cpp -- the `drainage` command-line driver on the GB300
// pipeline.  Accepts the reference's options (src/main.cpp:321-442) with
// the same meaning and defaults (src/framework/GlobalParameters.cpp:17-52):
//
//   --dem NAME (dem10)  --stream NAME (streams)  --dem-path DIR (DEM)
//   --stream-path DIR   (parsed; the reference reads streams from --dem-path)
//   --filter-type Gaussian|Exponential (Gaussian)
//   --practical-range F (60)  --error-mean F (0)  --error-standard-deviation F (1)
//   -i/--iterations N (10)    --gpu[=B]  --cpu[=B]
//   -o/--output-file FILE (.bin | .jpg)  --output-option end|frames
//
// Outputs: .bin = raw float32 counts; .jpg (the reference's default type) =
// the counts scaled to bytes as (uint8)rintf(255*((v-min)/max)) and written
// as the reference's jpge encoder writes them with its default parameters
// (quality 85; the same file bytes).
//
// Additive options: --seed N (default: the current time, like the
// reference's time(NULL)+iteration seeding), --bevel-radius N (2; the
// reference has no flag for it), --no-graphs, --fill cpu|exact (cpu: the
// reference CPU path's semantics, the default; exact: its GPU path's exact
// float fill, flat order and dead-end handling), --checkpoint FILE,
// --resume FILE, --batch K (realizations per batched step; 1).  Output
// files go to the
// working directory under the stem of -o (the reference keeps only the
// stem).  This driver runs on the GPU only; --cpu
// is refused rather than silently using another implementation.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>
#include "cageo.h"

namespace {

struct Options {
  std::string dem = "dem10", stream = "streams", dem_path = "DEM", stream_path = "DEM";
  std::string filter = "Gaussian", output_file, output_option, checkpoint, resume, fill = "cpu";
  float range = 60.0f, mean = 0.0f, sd = 1.0f;
  int iterations = 10, bevel = 2, batch = 1;
  bool gpu = true, cpu = false, graphs = true, have_seed = false;
  unsigned long long seed = 0;
};

void usage() {
  std::printf(
      "Options:\n"
      "  --help                       Produce help message\n"
      "  --dem arg (=dem10)           Name of the input DEM\n"
      "  --stream arg (=streams)      Name of the input stream network\n"
      "  --dem-path arg (=DEM)        Path to the input DEM\n"
      "  --stream-path arg (=DEM)     Path to the input stream network\n"
      "  --filter-type arg            Spatial autocorrelation model ('Gaussian' or 'Exponential')\n"
      "  --practical-range arg (=60)  Practical range of the autocorrelation model\n"
      "  --error-mean arg (=0)        Mean of the random field\n"
      "  --error-standard-deviation arg (=1)  Standard deviation of the random field\n"
      "  -i [ --iterations ] arg (=10) Number of Monte Carlo iterations\n"
      "  --gpu [=arg(=1)] (=1)        Run algorithm on GPU\n"
      "  --cpu [=arg(=1)] (=0)        Run algorithm on CPU (not available in this build)\n"
      "  -o [ --output-file ] arg     Write result into file (*.bin raw float32 counts, *.jpg image)\n"
      "  --output-option arg          end | frames\n"
      "  --seed arg                   Noise seed (default: current time)\n"
      "  --bevel-radius arg (=2)      Stream burning bevel radius (1..5)\n"
      "  --no-graphs                  Launch kernels directly instead of a CUDA graph\n"
      "  --fill arg (=cpu)            cpu: CPU-path semantics; exact: GPU-path exact float fill\n"
      "  --checkpoint arg             Save counts + next realization here after each output\n"
      "  --resume arg                 Continue from a checkpoint (same grid and --seed)\n"
      "  --batch arg (=1)             Realizations per batched step (CPU-path fill; same results)\n");
}

bool parse_bool(const std::string& v) { return !(v == "0" || v == "false" || v == "off"); }

int parse(int argc, char** argv, Options* o) {
  for (int i = 1; i < argc; i++) {
    std::string a = argv[i], val;
    bool has_val = false;
    size_t eq = a.find('=');
    if (a.rfind("--", 0) == 0 && eq != std::string::npos) {
      val = a.substr(eq + 1);
      a = a.substr(0, eq);
      has_val = true;
    }
    auto next = [&](std::string* out) -> bool {
      if (has_val) { *out = val; return true; }
      if (i + 1 >= argc) { std::fprintf(stderr, "missing value for %s\n", a.c_str()); return false; }
      *out = argv[++i];
      return true;
    };
    std::string v;
    if (a == "--help") { usage(); std::exit(0); }
    else if (a == "--dem") { if (!next(&o->dem)) return 1; }
    else if (a == "--stream") { if (!next(&o->stream)) return 1; }
    else if (a == "--dem-path") { if (!next(&o->dem_path)) return 1; }
    else if (a == "--stream-path") { if (!next(&o->stream_path)) return 1; }
    else if (a == "--filter-type") { if (!next(&o->filter)) return 1; }
    else if (a == "--practical-range") { if (!next(&v)) return 1; o->range = std::strtof(v.c_str(), nullptr); }
    else if (a == "--error-mean") { if (!next(&v)) return 1; o->mean = std::strtof(v.c_str(), nullptr); }
    else if (a == "--error-standard-deviation") { if (!next(&v)) return 1; o->sd = std::strtof(v.c_str(), nullptr); }
    else if (a == "-i" || a == "--iterations") { if (!next(&v)) return 1; o->iterations = std::atoi(v.c_str()); }
    else if (a == "--gpu") { o->gpu = has_val ? parse_bool(val) : true; }
    else if (a == "--cpu") { o->cpu = has_val ? parse_bool(val) : true; }
    else if (a == "-o" || a == "--output-file") { if (!next(&o->output_file)) return 1; }
    else if (a == "--output-option") { if (!next(&o->output_option)) return 1; }
    else if (a == "--seed") { if (!next(&v)) return 1; o->seed = std::strtoull(v.c_str(), nullptr, 10); o->have_seed = true; }
    else if (a == "--bevel-radius") { if (!next(&v)) return 1; o->bevel = std::atoi(v.c_str()); }
    else if (a == "--no-graphs") { o->graphs = false; }
    else if (a == "--batch") { if (!next(&v)) return 1; o->batch = std::atoi(v.c_str()); }
    else if (a == "--fill") {
      if (!next(&o->fill)) return 1;
      if (o->fill != "cpu" && o->fill != "exact") {
        std::fprintf(stderr, "--fill must be 'cpu' or 'exact'\n");
        return 1;
      }
    }
    else if (a == "--checkpoint") { if (!next(&o->checkpoint)) return 1; }
    else if (a == "--resume") { if (!next(&o->resume)) return 1; }
    else { std::fprintf(stderr, "unrecognised option '%s'\n", argv[i]); return 1; }
  }
  return 0;
}

std::string stem_of(const std::string& path, std::string* ext) {
  size_t slash = path.find_last_of('/');
  std::string base = slash == std::string::npos ? path : path.substr(slash + 1);
  size_t dot = base.find_last_of('.');
  if (dot == std::string::npos || dot == 0) { *ext = ""; return base; }
  *ext = base.substr(dot);
  return base.substr(0, dot);
}

int fail(const char* what) {
  std::fprintf(stderr, "%s: %s\n", what, cageo_last_error_string());
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  Options o;
  if (parse(argc, argv, &o)) { usage(); return 1; }
  if (o.cpu) {
    std::fprintf(stderr, "This drainage build runs the pipeline on the GPU only (--cpu refused).\n");
    return 1;
  }
  enum { NONE, END, FRAMES } opt = NONE;
  std::string out_name = "result", ext = ".jpg";
  if (!o.output_file.empty()) {
    std::string s = stem_of(o.output_file, &ext);
    if (ext != ".bin" && ext != ".jpg" && !ext.empty()) {
      std::printf("Unknown output extension provided: %s. Exiting...\n", ext.c_str());
      return 1;
    }
    if (!s.empty()) out_name = s;
    opt = END;
  }
  if (!o.output_option.empty()) {
    if (o.output_option == "end") opt = END;
    else if (o.output_option == "frames") opt = FRAMES;
    else { std::printf("Unknown output option provided: %s. Exiting...\n", o.output_option.c_str()); return 1; }
  }
  const bool jpeg = ext != ".bin";  // ".jpg" or no extension, as in the reference
  int model;
  if (o.filter == "Gaussian") model = CAGEO_FILTER_GAUSSIAN;
  else if (o.filter == "Exponential") model = CAGEO_FILTER_EXPONENTIAL;
  else { std::printf("Unknown filter type provided: %s. Exiting...\n", o.filter.c_str()); return 1; }
  if (o.iterations < 0) {
    std::printf("The number of iterations (%d) must not be negative. Exiting...\n", o.iterations);
    return 1;
  }
  if (!(o.range > 0.0f)) {
    std::printf("The practical range must be a positive number. Exiting...\n");
    return 1;
  }
  if (o.bevel < 1 || o.bevel > 5) {
    std::printf("Bevel radius (%d) is outside 1..5 (MAX_BEVEL_RADIUS 5).\n", o.bevel);
    return 1;
  }
  // The reference reads both headers and rasters from --dem-path (src/main.cpp:87-88,168-177).
  cageo_raster_info di, si;
  if (cageo_read_header((o.dem_path + "/" + o.dem + ".hdr").c_str(), &di)) return fail("DEM header");
  if (cageo_read_header((o.dem_path + "/" + o.stream + ".hdr").c_str(), &si)) return fail("stream header");
  bool bad = false;
  if (di.ncols != si.ncols) { std::printf("The sizes of the DEM and stream data don't match! Exiting...\n"); bad = true; }
  if (di.cellsize != si.cellsize) { std::printf("The cell size of the DEM and stream data don't match! Exiting...\n"); bad = true; }
  if (di.nrows != si.nrows) { std::printf("The row counts of the DEM and stream data don't match! Exiting...\n"); bad = true; }
  if (bad) return 1;
  const int W = di.ncols, H = di.nrows;
  const size_t N = (size_t)W * H;
  std::vector<float> dem(N), streams(N), counts(N);
  std::vector<uint8_t> image(jpeg ? N : 0);
  if (cageo_read_raster((o.dem_path + "/" + o.dem + ".bin").c_str(), dem.data(), N)) return fail("DEM raster");
  if (cageo_read_raster((o.dem_path + "/" + o.stream + ".bin").c_str(), streams.data(), N)) return fail("stream raster");
  const int r = cageo_filter_radius(o.range, di.cellsize);
  std::printf("DEM size: %d x %d\n", W, H);
  std::printf("Kernel size: %d x %d (%s)\n\n", 2 * r + 1, model == CAGEO_FILTER_GAUSSIAN ? 1 : 2 * r + 1,
              o.filter.c_str());
  cageo_pipeline_config cfg{};
  cfg.width = W;
  cfg.height = H;
  cfg.cell_size = di.cellsize;
  cfg.filter_model = model;
  cfg.practical_range = o.range;
  cfg.error_mean = o.mean;
  cfg.error_stddev = o.sd;
  cfg.bevel_radius = o.bevel;
  cfg.nodata_dem = di.nodata_value;
  cfg.nodata_stream = si.nodata_value;
  cfg.seed = o.have_seed ? o.seed : (unsigned long long)std::time(nullptr);
  cfg.use_graphs = o.graphs ? 1 : 0;
  cfg.fill_mode = o.fill == "exact" ? CAGEO_FILL_EXACT : CAGEO_FILL_CPU_COMPAT;
  std::printf("Seed: %llu\n", (unsigned long long)cfg.seed);
  cageo_pipeline* p = nullptr;
  if (cageo_pipeline_create(&p, &cfg, dem.data(), streams.data())) return fail("pipeline");
  if (o.batch != 1 && cageo_pipeline_set_batch(p, o.batch)) {
    cageo_pipeline_destroy(p);
    return fail("batch");
  }
  int start = 0;
  if (!o.resume.empty()) {
    uint32_t nxt = 0;
    if (cageo_pipeline_load(p, o.resume.c_str(), &nxt)) { cageo_pipeline_destroy(p); return fail("resume"); }
    start = (int)nxt;
    if (nxt > (uint32_t)o.iterations) {
      std::printf("The checkpoint %s already holds %u realizations, more than --iterations (%d). "
                  "Exiting...\n", o.resume.c_str(), nxt, o.iterations);
      cageo_pipeline_destroy(p);
      return 1;
    }
    std::printf("Resuming at realization %d\n", start);
  }
  // The END output (or the frame of realization it - 1): false on failure.
  auto write_output = [&](int it) {
    char name[4096];
    const char* suffix = jpeg ? ".jpg" : ".bin";
    if (opt == FRAMES) std::snprintf(name, sizeof(name), "%s_%04d%s", out_name.c_str(), it - 1, suffix);
    else std::snprintf(name, sizeof(name), "%s%s", out_name.c_str(), suffix);
    if (jpeg) {
      if (cageo_pipeline_counts_bytes(p, image.data())) return fail("counts") == 0;
      if (cageo_write_jpeg(name, image.data(), W, H, 85)) return fail("output") == 0;
    } else {
      if (cageo_pipeline_counts(p, counts.data())) return fail("counts") == 0;
      if (cageo_write_raster(name, counts.data(), N)) return fail("output") == 0;
    }
    return true;
  };
  auto t0 = std::chrono::steady_clock::now();
  for (int it = start; it < o.iterations;) {
    // One realization per call when every realization is written or saved.
    const int batch = (opt == FRAMES || !o.checkpoint.empty()) ? 1 : o.iterations - it;
    if (cageo_pipeline_run(p, (uint32_t)it, batch)) { cageo_pipeline_destroy(p); return fail("realization"); }
    it += batch;
    if (!o.checkpoint.empty() && cageo_pipeline_save(p, o.checkpoint.c_str(), (uint32_t)it)) {
      cageo_pipeline_destroy(p);
      return fail("checkpoint");
    }
    if (((opt == END && it == o.iterations) || opt == FRAMES) && !write_output(it)) {
      cageo_pipeline_destroy(p);
      return 1;
    }
  }
  // A resumed run with nothing left to do still writes the END output.
  if (opt == END && start == o.iterations && !write_output(start)) {
    cageo_pipeline_destroy(p);
    return 1;
  }
  double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  int64_t st[5] = {0};
  cageo_pipeline_stats(p, st, 5);
  const int done = o.iterations - start;
  std::fprintf(stderr, "\n***********\n\n%d realizations in %.3f s: %.3f realizations/s, %.3e cells/s\n",
               done, sec, done > 0 ? done / sec : 0.0, done > 0 ? done * (double)N / sec : 0.0);
  std::fprintf(stderr, "last realization: fill passes %lld, phases %lld, flat layers %lld\n",
               (long long)st[0], (long long)st[1], (long long)st[2]);
  cageo_pipeline_destroy(p);
  return 0;
}
