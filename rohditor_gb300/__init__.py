"""GB300 (sm_103a) sensor-development library: the C ABI in include/rd_gpu.h,
built from csrc/ into _lib/librd_gpu.so, with a host-side mirror of the
reference's `rohditor-gpu` processor interface."""

from .processor import (CaptureContract, capture_ceilings, ColorContract, Device, GamutDiagnostics, GpuBase, GpuDevelopedSource,
                        GpuPreviewError, GpuPreviewProcessor, GpuSensorProcessor, GpuSpatialProcessor, Histogram, JpegEncoder, launch_shape,
                        OpticsExecution, OutputSpec, PngEncoder, RlLaunchShape, SensorDescription, Stages, clip_levels,
                        light_tone_lut, opposed_levels, rl_launch_shape, standard_base_lut)

__all__ = [
    "CaptureContract", "capture_ceilings", "ColorContract", "Device", "GamutDiagnostics", "GpuBase", "GpuDevelopedSource", "GpuPreviewError",
    "GpuPreviewProcessor", "GpuSensorProcessor", "GpuSpatialProcessor", "Histogram", "JpegEncoder", "launch_shape", "OpticsExecution",
    "OutputSpec", "PngEncoder", "RlLaunchShape", "SensorDescription", "Stages", "clip_levels", "light_tone_lut", "opposed_levels", "rl_launch_shape",
    "standard_base_lut",
]
