"""GB300-native (sm_103a) KMeans Lloyd path, a drop-in for ferrolearn-cluster's KMeans.

The compute runs in hand-written CUDA kernels inside the in-tree library
_build/libferrokmeans.so, reached through its C ABI (include/ferrokmeans.h).
This package is the host-side mirror of the reference's KMeans API (and of
MiniBatchKMeans and BisectingKMeans, built on the same direct-form kernels).
"""
from .kmeans import (  # noqa: F401
    MIXED_BF16, MIXED_FP8, PLAIN, REDUCE_F64, REDUCE_REFERENCE, Context, CudaError, DeviceOutOfMemory, DeviceTimeout,
    FerroError, FittedKMeans, InsufficientSamples, InvalidParameter, KMeans, NullPointer, NumericalInstability,
    ShapeMismatch, Unsupported, default_context, draws, fit_batched, kmeans_plus_plus, lloyd_step)
from .minibatch import FittedMiniBatchKMeans, MiniBatchKMeans, minibatch_batch_indices  # noqa: F401
from .bisecting import BisectingKMeans, FittedBisectingKMeans  # noqa: F401

__version__ = "0.1.0"
