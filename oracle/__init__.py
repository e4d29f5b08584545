"""CPU oracle for the PCISPH time step (test infrastructure, never product code).

``oracle.oracle`` wraps the C++ restatement in ``pcisph_oracle.cpp`` (FP32 and
FP64); ``oracle.reference`` wraps the reference's own OpenCL kernels compiled on
the host (``build_ref.sh`` -> ``_ref/``), which exists only where the reference
sources are present and is used to generate and check golden vectors.
"""
