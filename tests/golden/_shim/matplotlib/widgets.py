"""Headless stand-in for matplotlib.widgets (import-time names only)."""


class AxesWidget:
    pass


class Slider(AxesWidget):
    pass


class RadioButtons(AxesWidget):
    pass


class RangeSlider(AxesWidget):
    pass
