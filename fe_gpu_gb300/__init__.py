"""fe_gpu_gb300: GB300-native (sm_103a) estimation core for high-dimensional
fixed-effects regressions, behind the C ABI of libfegb.so."""
from ._native import FeGpuError, library_path
from .bin_io import fe_dataset_header, fe_host_arrays, load_dataset_from_file, write_dataset
from .estimator import (DeviceBuffer, build_cluster_ids, compute_fe_group_sizes, fe_estimation_result, fe_gpu_estimate,
                        fe_gpu_estimate_device, fe_gpu_within_transform, fe_gpu_within_transform_device,
                        fe_runtime_config, init_default_config)

__all__ = [
    "FeGpuError", "library_path", "fe_dataset_header", "fe_host_arrays", "load_dataset_from_file", "write_dataset",
    "DeviceBuffer", "build_cluster_ids", "compute_fe_group_sizes", "fe_estimation_result", "fe_gpu_estimate",
    "fe_gpu_estimate_device", "fe_gpu_within_transform", "fe_gpu_within_transform_device", "fe_runtime_config",
    "init_default_config",
]
