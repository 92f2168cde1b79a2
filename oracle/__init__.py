"""CPU oracles for the GPU library (test infrastructure only).

``oracle.oracle.Port`` wraps ``oracle/liboracle.so``, a plain-C restatement of the
reference's hot path; ``oracle.oracle.Ref`` wraps ``oracle/_ref/libdsref.so``, the
unmodified reference compiled from its own sources (only where they exist).
The product never imports this package.
"""
