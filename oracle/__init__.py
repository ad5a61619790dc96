"""CPU oracle of the reference APIC/FLIP step — test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, as the checker and the timed CPU baseline; the product never imports
it.  Parity is unpinned: the reference has no tests or golden vectors and its
Rust toolchain is absent, so the restatement (apic_oracle.cpp) is checked
against hand-derived known answers and the GPU, not the reference's outputs.
"""
