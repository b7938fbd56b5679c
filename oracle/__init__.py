"""Oracle: FP64 CPU restatement of Spinach's static powder-FID path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (``spinach_gb300``) imports
this package.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it, and
there only as the checker or as the timed CPU baseline, never as the thing
measured on the GPU.

Parity pinning: the reference is MATLAB and cannot run in this environment.
The restatement is pinned against the closed-form expectations of the
reference's own tests (tests/kernel/*.m in the reference; each pin is cited in
tests/test_oracle_*.py) and against an independent Zeeman-basis Liouville model
(``oracle.kron_model``) that shares no code with the spherical-tensor path.
The multi-spin powder FID itself is not pinned by any reference test; beyond
the analytic cases parity is oracle-vs-GPU.
"""
