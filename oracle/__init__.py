"""CPU oracles for the binary-sparse 2-D R2C FFT -- TEST INFRASTRUCTURE ONLY.

Nothing in the cuspfft_gb300 package imports this package.  It is used by
tests/, by __graft_entry__.smoke() as the checker, and by bench.py for the
accuracy column and the CPU baseline leg.

  fp64.py      double-precision DFT of the binary matrix (exact integer phases)
  ref_port.py  restatement of the reference's FP32 GPU method and CPU path
  ref_shim.cu  + build_ref.sh : the reference's own host code, compiled from
               its sources into oracle/_ref/ where they are present
"""
