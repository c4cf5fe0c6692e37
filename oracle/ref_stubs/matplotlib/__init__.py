"""Import-time stand-in for matplotlib, used only when the reference CyLag
build is imported as a test oracle (plotting and the matplotlib trifinder are
not on the per-particle step; cylag/extra/plot_utils.pyx:23-25,
cylag/core/eulerian_field_set.pyx:23)."""


def rc(*args, **kwargs):
    return None


def use(*args, **kwargs):
    return None
