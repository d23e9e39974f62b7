"""GB300-native party-B scoring for secure genotype imputation.

A drop-in for the cloud step of ssmiler/idash2019_2 (cloud_compute_score,
eval/idash.cpp:763-848): integer-weighted sums of encrypted one-hot tag-SNP
ciphertexts (Torus32 TRLWE / LWE) plus a bias, exact mod 2^32, computed by
hand-written sm_103a CUDA kernels behind the C ABI in include/idash_gpu.h.

Build with idash2019_2_gb300.build.build() (or __graft_entry__.build()).
"""
from .build import build  # noqa: F401

__all__ = ["build"]
