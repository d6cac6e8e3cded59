"""ORACLE: CPU restatement of mom25d\x27s sweep path (test infrastructure only)."""
