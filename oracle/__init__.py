"""Oracle for the meshless Laguerre cell path -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg;
never by the product (geogram_gb300)."""
