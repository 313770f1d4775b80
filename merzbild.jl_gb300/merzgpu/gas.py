"""Gas data used by the benchmark configurations and tests.

Values are the ones Merzbild.jl loads from its data files (data/particles.toml,
data/vhs.toml, data/pseudo_maxwell.toml) and asserts in test/runtests.jl:85-102.
Use load_species_data / load_interaction_data to read TOML files instead.
"""
AR_MASS = 66.3e-27
HE_MASS = 6.65e-27

# "A,B": (vhs_d, vhs_o, vhs_Tref)
VHS = {"Ar,Ar": (4.11e-10, 0.81, 273.0), "Ar,He": (3.25e-10, 0.735, 273.0), "He,He": (2.33e-10, 0.66, 273.0)}
PSEUDO_MAXWELL = {"Ar,Ar": (4.11e-10, 1.0, 273.0), "Ar,He": (3.25e-10, 1.0, 273.0), "He,He": (2.33e-10, 1.0, 273.0)}
