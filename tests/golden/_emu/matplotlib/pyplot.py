"""Empty stand-in for matplotlib.pyplot (fixture generation only; never called)."""
