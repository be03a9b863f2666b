"""Drop-in for the reference's adi/ package (adi/rhs.py, adi/transpose.py)."""
