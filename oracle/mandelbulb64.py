"""Whether a Mandelbulb escape iteration is determined at float32 precision
(test infrastructure only).

The escape iteration of pos -> pos^10 + c (Benchmarks/Mandlebulb/Worklets.h:
65-109) is chaotic near the fractal's boundary: the power map grows
differences about tenfold a step, tan(10 phi) has poles, and the escape test
compares |pos|^2 with 2.  Two float32 implementations whose atan2, pow, sin,
tan and cos round differently in the last place therefore disagree on some
points.  A point's count is called determined when an ensemble of FP64
orbits of the same float32 coordinate agrees on it: the exact orbit, the
orbit with every intermediate rounded to float32, and `trials` orbits in
which every intermediate (the arguments of the trigonometric functions
included) is perturbed by a random relative error of at most `ulps` float32
units.  Where the ensemble disagrees, float32 arithmetic does not determine
the count."""
import numpy as np

U = 2.0 ** -24


def _escape(c, rng=None, ulps=4.0, f32=False):
    def q(x):
        if f32:
            x = x.astype(np.float32).astype(np.float64)
        if rng is not None:
            x = x * (1.0 + rng.uniform(-ulps, ulps, size=x.shape) * U)
        return x

    c = np.asarray(c, np.float64)
    pos = c.copy()
    esc = np.where(q((pos ** 2).sum(1)) > 2, 0, -1)
    with np.errstate(all="ignore"):
        for i in range(1, 35):
            live = esc < 0
            sq = q((pos ** 2).sum(1))
            t = q(np.sqrt(q(pos[:, 0] ** 2 + pos[:, 1] ** 2)))
            th = q(10 * q(np.arctan2(t, pos[:, 2])))
            ph = q(10 * q(np.arctan2(pos[:, 1], pos[:, 2])))
            pr = q(sq ** 5)
            s_th = q(np.sin(th))
            nxt = np.stack([q(pr * q(s_th * q(np.tan(ph)))), q(pr * q(s_th * q(np.sin(ph)))),
                            q(pr * q(np.cos(th)))], 1)
            pos = np.where(live[:, None], q(nxt + c), pos)
            esc = np.where(live & (q((pos ** 2).sum(1)) > 2), i, esc)
    return np.where(esc < 0, 35, esc)


def ensemble(c, trials=8, ulps=4.0, seed=0):
    """Escape counts [2 + trials, n] of the ensemble for float32 coordinates
    c [n, 3]: exact, float32-rounded, then the perturbed orbits."""
    rows = [_escape(c), _escape(c, f32=True)]
    rows += [_escape(c, np.random.default_rng(seed + k), ulps) for k in range(trials)]
    return np.stack(rows, 0)


def determined(E):
    """Points whose ensemble agrees, and that count."""
    return (E == E[0]).all(0), E[0]
