"""CPU oracle of the Elfel.jl assembly + solve path (test infrastructure only)."""
