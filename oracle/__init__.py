"""CPU restatement of the reference step: the checker and the CPU baseline.

Test infrastructure only; the product path (swe_fvm_gb300) never imports it.
"""
