// ref_harness.cpp -- drives the drainage reference's own CPU stage templates
// (compiled from the reference sources, not copied) behind the same C
// signatures as oracle/cageo_oracle.cpp, so tests can compare the two.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile into oracle/_ref/ on a
// machine where the reference sources exist; it cannot run where they were
// not compiled.  Used to generate the golden fixtures in tests/golden/ and to
// pin the CPU restatement.
//
// What is injected instead of called (the reference libraries that build the
// filter and the noise are not available here):
//  * the convolution filter: a subclass sets the protected filter members of
//    ConvolutionAlgorithm_CPU_OpenMP (src/convolution/ConvolutionAlgorithm.h:208-221);
//  * the noise: written straight into the RandomField buffer, as
//    RandomFieldAlgorithm_CPU_OpenMP::generateRandomField would
//    (src/randomfield/RandomFieldAlgorithmCPUOpenMP.h:47-76).
#include <cstdio>
#include <cstring>
#include <cstdint>

#include "AbstractFactory.h"
#include "GlobalParameters.h"
#include "RasterDEM.h"
#include "StreamData.h"
#include "RandomFieldClass.h"
#include "ConvolutionAlgorithmCPUOpenMP.h"
#include "RealisticDemAlgorithm.h"
#include "StreamBurningAlgorithmCPUOpenMP.h"
#include "PitFillingAlgorithmCPUOpenMP.h"
#include "FlowRoutingAlgorithmCPUOpenMP.h"
#include "FlowTracingAlgorithmCPUOpenMP.h"
#include "CatchmentBorderAlgorithmCPUOpenMP.h"
#include "FlowDirClass.h"
#include "FlowTraceDataClass.h"
#include "CatchmentBorderClass.h"
#include "ToByteArrayAlgorithm.h"
#include "ToByteArrayAlgorithmCPUOpenMP.h"
#include "jpge.h"

namespace {

struct Setup {
  Setup() { AbstractFactory::defaultImpl = AbstractFactory::CPU; }
} g_setup;

// Exposes the protected filter state (the reference builds it with FFTW and
// Eigen in ConvolutionAlgorithm.cpp, which are not available).
class InjectedConvolution : public ConvolutionAlgorithm_CPU_OpenMP<float> {
 public:
  void inject(const float* taps, int count, int radius, FilterModel model) {
    this->filterRadius = radius;
    this->filterModel = model;
    this->filter = ManagedDataFactory::create<filter_t>(count, HOST);
    this->filter->allocateData();
    std::memcpy(this->filter->getData(), taps, sizeof(float) * count);
  }
};

// The reference allocates its 121-entry search-offset table with new[]
// (src/streamburning/StreamBurningAlgorithm.h:121-128,
// src/framework/ManagedData.h:638) and its generator writes only the offsets
// within the bevel radius (:143-166); the burn loop stops at the first (0,0)
// entry (src/streamburning/StreamBurningAlgorithmCPUOpenMP.h:57-60).  The
// entries after the last offset are therefore whatever the heap held, and in
// a long-lived process the loop can run on into stale offsets.  This subclass
// allocates the table itself, zero-filled (what fresh memory holds), and lets
// the reference's own generator write the offsets; execute() then finds the
// table present and uses it.
class ZeroTailBurning : public StreamBurningAlgorithm_CPU_OpenMP<float, float> {
 public:
  explicit ZeroTailBurning(int bevel) {
    this->setBevelRadius(bevel);
    this->circularSearchArray =
        ManagedDataFactory::create<CoordOffset>(MAX_CIRCULAR_ARRAY_SIZE, HOST);
    this->circularSearchArray->allocateData();
    std::memset((void*)this->circularSearchArray->getData(), 0,
                sizeof(CoordOffset) * MAX_CIRCULAR_ARRAY_SIZE);
    this->generateCircularSearchArray(this->circularSearchArray->getData(), bevel);
  }
};

// The reference allocates each realization's border grid with new[] and
// writes only its 1s (src/catchmentborder/CatchmentBorderAlgorithm.h:64-66,
// src/catchmentborder/CatchmentBorderAlgorithmCPUOpenMP.h:30-82,
// src/framework/ManagedData.h:638); the other cells are whatever the heap
// held.  This subclass zeroes the grid (what fresh memory holds) before the
// reference's own extraction runs on it.
class ZeroedBorder
    : public CatchmentBorderAlgorithm_CPU_OpenMP<CatchmentBorderType, FlowTraceDataType> {
 public:
  void performExtractDrainageBorder(CatchmentBorderClass<CatchmentBorderType>* border,
                                    FlowTraceDataClass<FlowTraceDataType>* trace) {
    border->toHost();
    std::memset((void*)border->getData(), 0,
                sizeof(CatchmentBorderType) * (size_t)border->width * border->height);
    CatchmentBorderAlgorithm_CPU_OpenMP<CatchmentBorderType,
                                        FlowTraceDataType>::performExtractDrainageBorder(border,
                                                                                         trace);
  }
};

template <typename G>
void load(G& g, const void* src, size_t bytes) {
  std::memcpy((void*)g.getData(), src, bytes);
}

}  // namespace

extern "C" {

int ref_convolve(const float* in, float* out, int W, int H, const float* filt,
                 int r, int model) {
  RandomField_t field(W, H, HOST);
  load(field, in, sizeof(float) * W * H);
  InjectedConvolution conv;
  int L = 2 * r + 1;
  conv.inject(filt, model == 1 ? L : L * L, r, model == 1 ? GAUSSIAN : EXPONENTIAL);
  conv.execute(&field);
  std::memcpy(out, field.getData(), sizeof(float) * W * H);
  return 0;
}

void ref_realistic_dem(const float* dem, float* field, int W, int H,
                       float nodata_dem) {
  G::noDataValueDEM = nodata_dem;
  RasterDEM_t d(W, H, HOST);
  load(d, dem, sizeof(float) * W * H);
  RandomField_t f(W, H, HOST);
  load(f, field, sizeof(float) * W * H);
  RealisticDemAlgorithm_t alg;
  alg.execute(&d, &f, (RasterDEM_t*)&f);
  std::memcpy(field, f.getData(), sizeof(float) * W * H);
}

void ref_stream_burn(float* dem, const float* streams, int W, int H, int bevel,
                     float nodata_dem, float nodata_stream) {
  RasterDEM_t d(W, H, HOST);
  load(d, dem, sizeof(float) * W * H);
  StreamData_t s(d, AS_TEMPLATE);
  load(s, streams, sizeof(float) * W * H);
  ZeroTailBurning alg(bevel);
  alg.setNoDataValueDEM(nodata_dem);
  alg.setNoDataValueStream(nodata_stream);
  alg.execute(&d, &s);
  std::memcpy(dem, d.getData(), sizeof(float) * W * H);
}

void ref_pitfill(float* dem, float* filled, int W, int H, float nodata) {
  RasterDEM_t d(W, H, HOST);
  load(d, dem, sizeof(float) * W * H);
  RasterDEM_t f(W, H, HOST);
  PitFillingAlgorithm_CPU_OpenMP<float> alg;
  alg.setNoDataValueDem(nodata);
  alg.execute(&f, &d);
  std::memcpy(dem, d.getData(), sizeof(float) * W * H);
  std::memcpy(filled, f.getData(), sizeof(float) * W * H);
}

void ref_flow_route(const float* dem, int8_t* dir, int* flatdist, int W, int H) {
  RasterDEM_t d(W, H, HOST);
  load(d, dem, sizeof(float) * W * H);
  FlowDir_t fd(W, H, HOST);
  FlowRoutingAlgorithm_CPU_OpenMP<FlowDirDataType, DemData> alg;
  alg.execute(&fd, &d);
  std::memcpy(dir, fd.getData(), 2 * (size_t)W * H);
  (void)flatdist;  // the flat-distance grid is internal to execute()
}

void ref_flow_trace(const int8_t* dir, const float* streams, int* label, int W,
                    int H) {
  FlowDir_t fd(W, H, HOST);
  load(fd, dir, 2 * (size_t)W * H);
  RasterDEM_t model(W, H, HOST);
  StreamData_t s(model, AS_TEMPLATE);
  load(s, streams, sizeof(float) * W * H);
  FlowTraceData_t t(W, H, HOST);
  FlowTracingAlgorithm_CPU_OpenMP<FlowTraceDataType, FlowDirDataType, DemData> alg;
  alg.execute(&t, &fd, &s);
  std::memcpy(label, t.getData(), sizeof(int) * (size_t)W * H);
  std::fflush(stdout);  // the walk's "Infinite loop?" notes go out with this call's output
}

void ref_border_accumulate(const int* label, float* mc, int W, int H) {
  FlowTraceData_t t(W, H, HOST);
  load(t, label, sizeof(int) * (size_t)W * H);
  CatchmentBorder_t m(t, AS_TEMPLATE);
  load(m, mc, sizeof(float) * (size_t)W * H);
  ZeroedBorder alg;
  alg.execute(&m, &t);
  std::memcpy(mc, m.getData(), sizeof(float) * (size_t)W * H);
}

// The JPEG output: the count grid as bytes (ToByteArrayAlgorithm on the
// CPU, src/utils/tobytearray/ToByteArrayAlgorithmCPUOpenMP.h:33-52), then
// the jpge encoder on one channel with its default parameters, as the
// driver calls both (src/main.cpp:258-271); `quality` replaces the
// default 85 when it is not 0.
void ref_to_bytes(const float* mc, uint8_t* out, int W, int H) {
  CellGrid<float> m(W, H, HOST);
  load(m, mc, sizeof(float) * (size_t)W * H);
  CellGrid<Byte_t> bytes(m, AS_TEMPLATE);
  ToByteArrayAlgorithm_CPU_OpenMP<float> alg;
  alg.execute(&bytes, &m);
  std::memcpy(out, bytes.getData(), (size_t)W * H);
}

int ref_write_jpeg(const char* path, const uint8_t* img, int W, int H, int quality) {
  jpge::params p;
  if (quality) p.m_quality = quality;
  return jpge::compress_image_to_jpeg_file(path, W, H, 1, (const jpge::uint8*)img, p) ? 0 : 1;
}

}  // extern "C"
