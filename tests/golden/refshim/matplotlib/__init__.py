"""Empty stand-in: ceviche imports matplotlib.pylab at module level for plots only."""
