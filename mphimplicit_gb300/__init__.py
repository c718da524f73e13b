"""GB300-native MPH-I time-step engine (Moving Particle Hydrodynamics for
incompressible flows, implicit)."""
