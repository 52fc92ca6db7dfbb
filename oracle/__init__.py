"""The oracle: CPU restatement of the DeepDRR projector and a driver for the reference kernel.

TEST INFRASTRUCTURE ONLY. Imported by the tests, by ``__graft_entry__.smoke()`` and by the
CPU-baseline leg of ``bench.py``; never by the ``deepdrr_gb300`` package.
"""
