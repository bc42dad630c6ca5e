"""CPU restatement of the reference step (the checker and the CPU baseline) and
the reference's own solver built from its sources (the restatement's pin).

Test infrastructure only; the product path (swe_fvm_gb300) never imports it.
"""
