"""CPU oracle for the MDACP Lennard-Jones hot path (test infrastructure only).

`oracle.port` wraps the C restatement (mdacp_oracle.c); `oracle.refrun` runs
the reference itself, built from its own sources by build_ref.sh.  Only the
tests, the smoke check and the benchmark's CPU-baseline leg import this
package; the GPU library never does.
"""
