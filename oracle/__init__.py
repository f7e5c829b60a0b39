"""Oracle: TEST INFRASTRUCTURE ONLY.

CPU restatements of the reference's (sharhar/vkdispatch) FFT, FFT-convolution
and reduction algorithms, plus the FP64 numpy.fft accuracy oracle.  Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import
this package, and only as the checker or the timed CPU baseline -- never as
part of the product path (vkdispatch_gb300 has no CPU fallback).
"""
