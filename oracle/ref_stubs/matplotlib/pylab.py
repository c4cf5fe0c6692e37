"""Empty pylab stand-in (plotting is not on the per-particle step)."""
