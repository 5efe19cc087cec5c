"""CPU oracle and reference-kernel harness for the IronClust hot path.

Test infrastructure only: imported by tests/, the smoke check and the CPU
baseline of bench.py as the checker, never by the shipped library.
"""
