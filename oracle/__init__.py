"""Test oracle for pmdas_gb300 (CPU restatement + reference harness).  Test infrastructure only."""
