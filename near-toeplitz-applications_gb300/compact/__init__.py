"""Drop-in for the reference's compact/ package (compact/rhs.py, compact/permute.py)."""
