"""CPU oracle for the chunk-extraction hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
use this package, and only as the checker / the timed CPU baseline.  The product
(``binarymeshfitting_gb300``) never imports it.

``oracle.ref`` wraps the reference's own compiled code (oracle/_ref, built only
where the reference sources are present); ``oracle.cpu`` wraps the C
restatement (oracle/_build/libbmf_oracle.so), which runs anywhere.
"""
