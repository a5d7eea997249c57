"""GB300-native read-to-contig Smith-Waterman: the alignment hot path of MHM2's klign.

The product is libmhsw.so (CUDA kernels for sm_103a + host driver, C ABI in
include/mhsw.h).  This package builds it (build.py), binds it (driver.py: a Python
mirror of adept_sw::GPUDriver) and generates the seeded workloads (workloads.py).
"""
from .driver import (FORM_BATCHED, FORM_PLAIN, ORIENT_KLIGN, ORIENT_REF_IS_A, GPUDriver, Pairs,  # noqa: F401
                     get_avail_gpu_mem_per_rank, get_device_name, get_num_node_gpus, get_tot_gpu_mem,
                     initialize_gpu, load_library)
