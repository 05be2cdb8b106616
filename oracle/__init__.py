"""Test infrastructure: CPU oracle and reference-parity harness (never imported by the product)."""
