"""Host pose bookkeeping of the reference tracker restated for the tests.

apply_increment_ref_order restates PhotoTracker::applyIncrement
(phototracker.cpp:514-531) in Python floats in the reference's operation
order; tests/test_oracle_pin.py pins it bit for bit to the reference's own
code (oracle/_ref), and the GPU tests use it to check recon_track's global
pose.
"""
import numpy as np


def apply_increment_ref_order(T_host, G, Trel):
    """PhotoTracker::applyIncrement's arithmetic (phototracker.cpp:514-531) in
    Python floats, in the reference's operation order (invertRT4 and
    matrixMult4x4 of basic_math.cpp): returns the new host pose (float32,
    current -> reference) and global pose (float64)."""
    def inv(M):
        M = [float(v) for v in M]
        return [M[0], M[4], M[8], -(M[0] * M[3] + M[4] * M[7] + M[8] * M[11]),
                M[1], M[5], M[9], -(M[1] * M[3] + M[5] * M[7] + M[9] * M[11]),
                M[2], M[6], M[10], -(M[2] * M[3] + M[6] * M[7] + M[10] * M[11]),
                0.0, 0.0, 0.0, 1.0]

    def mul(A, B):
        return [A[r * 4] * B[c] + A[r * 4 + 1] * B[4 + c] + A[r * 4 + 2] * B[8 + c] + A[r * 4 + 3] * B[12 + c]
                for r in range(4) for c in range(4)]

    iTprev = inv(np.asarray(T_host, np.float32).reshape(16))
    Tdbl = inv(np.asarray(Trel, np.float32).reshape(16))
    T_new = np.asarray(Tdbl, np.float64).astype(np.float32)
    G_new = mul([float(v) for v in np.asarray(G, np.float64).reshape(16)], mul(iTprev, Tdbl))
    return T_new.reshape(4, 4), np.asarray(G_new, np.float64).reshape(4, 4)
