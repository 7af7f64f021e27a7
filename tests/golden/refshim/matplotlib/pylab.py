"""Empty stand-in for matplotlib.pylab (plotting is never called by the fixture script)."""
