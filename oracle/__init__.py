"""CPU oracle of the sDEM hot path: TEST INFRASTRUCTURE ONLY (tests/, smoke(),
bench.py's CPU-baseline leg).  The product never imports this package."""
