"""Recipe and driver that build the reference's own solver into oracle/_ref
(test infrastructure only)."""
