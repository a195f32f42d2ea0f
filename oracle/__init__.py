"""CPU oracle of the azplugins force-and-integrate path (test infrastructure only)."""
