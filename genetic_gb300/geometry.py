"""Integer cell windows on a periodic grid, as genetIC's Window<int> keeps them
(genetIC/src/simulation/window.hpp), for placing zoom grids around flagged cells."""


class Window:
    """A cuboid of cells [lower, upper) per axis on a periodic domain of `wrap` cells."""

    def __init__(self, wrap, lower, upper=None):
        self.wrap_length = int(wrap)
        self.lower = [int(v) for v in lower]
        self.upper = [int(v) + 1 for v in lower] if upper is None else [int(v) for v in upper]
        if upper is not None:
            self.wrap_corners()

    def wrap(self, v):
        if v < 0:
            v += self.wrap_length
        if v >= self.wrap_length:
            v -= self.wrap_length
        return v

    def wrap_corners(self):
        self.lower = [self.wrap(v) for v in self.lower]
        self.upper = [self.wrap(v - 1) + 1 for v in self.upper]

    @staticmethod
    def within_wrapped(lo, hi, v):
        if hi >= lo:
            return lo <= v < hi
        return v < hi or v >= lo

    def sizes(self):
        return [self.wrap(u - l - 1) + 1 for l, u in zip(self.lower, self.upper)]

    def maximum_dimension(self):
        return max(self.sizes())

    def centre(self):
        return [self.wrap(l + self.wrap(u - 1 - l) // 2) for l, u in zip(self.lower, self.upper)]

    def contains_axis(self, v, a):
        return self.within_wrapped(self.lower[a], self.upper[a], v)

    def expand_to_include(self, p):
        """Window::expandToInclude (window.hpp:177-199): per axis, move the nearer corner."""
        for a in range(3):
            lo, hi, v = self.lower[a], self.upper[a], p[a]
            if self.within_wrapped(lo, hi, v):
                continue
            size_lower = self.wrap(hi - v - 1) + 1
            size_upper = self.wrap(v + 1 - lo - 1) + 1
            can_lower = self.within_wrapped(v, hi, lo)
            can_upper = self.within_wrapped(lo, v + 1, hi - 1)
            if can_lower and (size_lower < size_upper or not can_upper):
                self.lower[a] = v
            else:
                self.upper[a] = v + 1

    def expand_symmetrically_to_size(self, n):
        """Window::expandSymmetricallyToSize (window.hpp:202-239), including its correction
        of the y axis against the old lower corner's z component."""
        old = list(self.lower)
        if n == self.wrap_length:
            self.lower, self.upper = [0, 0, 0], [n, n, n]
            return
        c = self.centre()
        self.lower = [self.wrap(v - n // 2) for v in c]
        if n % 2 == 0:
            self.upper = [self.wrap(v + n // 2 - 1) + 1 for v in c]
        else:
            self.upper = [self.wrap(v + n // 2) + 1 for v in c]
        if self.lower[0] > old[0]:
            self.lower[0] -= 1
            self.upper[0] -= 1
        if self.lower[1] > old[2]:
            self.lower[1] -= 1
            self.upper[1] -= 1
        if self.lower[2] > old[2]:
            self.lower[2] -= 1
            self.upper[2] -= 1

    def wrapped_offset(self, a, b):
        d = b - a
        if d < -self.wrap_length / 2:
            d += self.wrap_length
        if d > self.wrap_length / 2:
            d -= self.wrap_length
        return d

    def shift(self, d):
        self.lower = [l + s for l, s in zip(self.lower, d)]
        self.upper = [u + s for u, s in zip(self.upper, d)]
        self.wrap_corners()

    def move_into(self, other):
        """Window::moveInto (window.hpp:246-273): the smallest wrapped move that puts this
        window inside `other`."""
        move = [0, 0, 0]
        for a in range(3):
            if not other.contains_axis(self.lower[a], a):
                move[a] = self.wrapped_offset(self.lower[a], other.lower[a])
            if not other.contains_axis(self.upper[a] - 1, a):
                move[a] = self.wrapped_offset(self.upper[a], other.upper[a])
        self.shift(move)


def zoom_corner(flags, n_above, box_above, offset_above, periodic, zoomfac):
    """ICGenerator::initZoomGrid's placement (ic.hpp:398-476): the window of the flagged cells
    of the level above (ascending ids), grown symmetrically to n_above / zoomfac cells, moved
    inside the level above; returns its lower corner in that level's cells."""
    if len(flags) == 0:
        raise RuntimeError('Cannot initialise zoom without marking particles to be replaced')
    dx = box_above / n_above
    wrap = int(round(periodic / dx))

    def coord(c):
        c = int(c)
        return [c // (n_above * n_above), (c // n_above) % n_above, c % n_above]

    w = Window(wrap, coord(flags[0]))
    for c in flags:
        w.expand_to_include(coord(c))
    n_required = w.maximum_dimension()
    n_user = n_above // int(zoomfac)
    if n_required > n_user:
        raise RuntimeError('Zoom particles do not fit in specified sub-box. Decrease zoom, or choose different particles')
    if n_required < n_user:
        w.expand_symmetrically_to_size(n_user)
    corner = [int(round(o / dx)) for o in offset_above]
    above = Window(wrap, corner, [c + n_above for c in corner])
    w.shift(corner)
    w.move_into(above)
    w.shift([-c for c in corner])
    return w.lower
