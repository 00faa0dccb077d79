"""CPU oracle of the duct substep (test infrastructure; see ekref.h)."""
