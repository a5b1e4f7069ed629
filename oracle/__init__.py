"""TEST INFRASTRUCTURE — the CPU oracle (checker only; never imported by the product)."""
