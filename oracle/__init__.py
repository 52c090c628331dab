"""Test infrastructure only: CPU oracles for the propagator-contraction path.

Nothing in the product (``contract_gb300``) imports this package.  Only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use it, and only as the oracle the CUDA path is compared with.

Layers, from most to least independent of the reference's own code:

* ``gamma``          -- DeGrand-Rossi gamma basis built from the four gamma
                        matrices; index/phase tables derived from it.
* ``einsum_oracle``  -- FP64 numpy einsum restatement of every contraction
                        (the ``doc/contract.py`` / ``baryon_2pt.py:31-41``
                        index strings of CLQCD/contract).
* ``contract_oracle.c`` (``lib.py`` loads it) -- a plain-C FP64 restatement of
                        the reference's per-site algorithm (16 spin pairs,
                        epsilon-epsilon colour loop), OpenMP over sites.  It
                        is also the CPU baseline timed by ``bench.py``.
* ``Makefile`` + ``ref_shim/`` + ``ref_*.cpp`` -- compile the reference's own
                        ``*_local`` device functions as host C++ into
                        ``oracle/_ref/libcontract_ref.so`` (only where the
                        reference sources are present).  This pins the other
                        layers to the reference's arithmetic.
"""
