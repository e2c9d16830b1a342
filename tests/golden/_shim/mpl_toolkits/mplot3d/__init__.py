"""Headless stand-in for mpl_toolkits.mplot3d."""


class Axes3D:
    pass
