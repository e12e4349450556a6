"""GB300-native PAR2 recovery backend (par2cuda) and its host-side drivers.

The job stream runs a dozen or more CUDA streams side by side (copies, the
contraction, IFSC, several file MD5 launches of up to seconds each).  CUDA
maps streams onto CUDA_DEVICE_MAX_CONNECTIONS hardware queues, 8 by default,
and two streams that share a queue wait for each other's work in issue order:
a long MD5 launch then holds back a contraction or another MD5 launch queued
behind it.  Importing the package before the process creates its CUDA context
raises the default to 32 queues (a value set by the caller is kept).
"""
import os

os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
