// rocm_names.hpp — the reference's class names for the GB300 facades, so code
// written against DspSpectrum compiles unchanged against this library:
//   fft_processor::FFTProcessorROCm       (include/spectrum/fft_processor_rocm.hpp:53)
//   fft_processor::ComplexToMagPhaseROCm  (include/spectrum/complex_to_mag_phase_rocm.hpp:83)
//   antenna_fft::SpectrumProcessorROCm    (include/spectrum/processors/spectrum_processor_rocm.hpp:96)
//   antenna_fft::AllMaximaPipelineROCm    (include/spectrum/pipelines/all_maxima_pipeline_rocm.hpp:42)
// The one signature that differs: AllMaximaPipelineROCm(hipStream_t, IBackend*)
// becomes AllMaximaPipelineGB300(IBackend*) (the stream comes from the backend).
#pragma once

#include "spectrum_gb300/spectrum.hpp"

namespace fft_processor {
using FFTProcessorROCm = FFTProcessorGB300;
using ComplexToMagPhaseROCm = ComplexToMagPhaseGB300;
}  // namespace fft_processor

namespace antenna_fft {
using SpectrumProcessorROCm = SpectrumProcessorGB300;
using AllMaximaPipelineROCm = AllMaximaPipelineGB300;
}  // namespace antenna_fft
