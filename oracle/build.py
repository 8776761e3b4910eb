"""Build recipe for the C oracle (test infrastructure only).

Compiles ``oracle/cd_oracle.c`` into ``oracle/liboracle.so`` with strict IEEE
float64 semantics: no fused multiply-add contraction, no fast-math, so each
operation rounds exactly like the reference's numba/numpy arithmetic.
OpenMP is used only by the agent-parallel variant of the timed CPU baseline.
The shared elementary functions (crowddynamics_gb300/csrc/cd_math.h) are
included so the oracle can round exactly like the device when asked to.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, 'cd_oracle.c')
MATH = os.path.join(os.path.dirname(HERE), 'crowddynamics_gb300', 'csrc', 'cd_math.h')
LIB = os.path.join(HERE, 'liboracle.so')


def build(force=False, verbose=False):
    """Compile the oracle if the library is missing or older than its source."""
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(MATH))):
        return LIB
    cmd = ['gcc', '-O2', '-std=c11', '-ffp-contract=off', '-fno-fast-math',
           '-fPIC', '-shared', '-fopenmp', '-I', os.path.dirname(MATH), SRC, '-o', LIB + '.tmp', '-lm']
    if verbose:
        print(' '.join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + '.tmp', LIB)
    return LIB


if __name__ == '__main__':
    build(force='--force' in sys.argv, verbose=True)
