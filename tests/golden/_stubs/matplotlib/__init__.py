"""Empty stand-in for matplotlib so that plotting modules import."""
