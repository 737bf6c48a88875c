"""CPU oracle for distance3d_gb300 (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this
package; the product never does.
"""
