"""CPU oracle for the greedy sparse-recovery hot path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use this
package.  The product (gaga_gb300) never imports it.
"""
