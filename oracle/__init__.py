"""CPU oracle for the tiled Cholesky / LU / QR hot path (test infrastructure only)."""
