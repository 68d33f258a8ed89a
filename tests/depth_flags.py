"""Classification of the depth filter's flag disagreements between a float run and the FP64 oracle
(test infrastructure, used by test_depth_flags.py and test_gpu_depth.py).

A pixel "disagrees" when its validity or blacklist count differs between the two runs.  Both runs
of the oracle record every threshold decision they take (oracle/lsdo_depth.cpp, decision trace):
the compared quantity q, its threshold and the branch taken.  For each disagreeing pixel the two
traces are walked in step until the first record where the runs branch differently; that record
explains the pixel when

* it straddles its threshold by a rounding-sized margin: the float run's quantity lies within
  `tol` (relative, 2e-3: the SSD of five differences of bilinear samples carries the rounding of
  the search start, itself fused from several observations) of the threshold, and within `tol` of
  the FP64 run's quantity (so the two runs
  computed the same number up to rounding and fell on opposite sides); or
* it is a decision on another pixel's state (a neighbour's hypothesis in regularisation, a source
  pixel of propagation) and that other pixel's own trace diverged at an earlier stage, and is
  itself explained; or
* for an argmin (the best 5-sample SSD window, the z-buffer winner of propagation): the two
  candidates' values lie within `tol` of each other in the float run.

Stages: 0 observeDepth (per keyframe pixel and reference), 1 the update's regularisation, 2
propagation (keyed by the old keyframe pixel), 3 the new keyframe's regularisation.  Decision ids
follow oracle/lsdo_depth.cpp (DecisionId).
"""
from __future__ import annotations

import numpy as np

import lsdo

# DecisionId values of oracle/lsdo_depth.cpp
D = dict(GRAD=1, EPL=2, COS=3, AZ=4, EPLLEN=5, RANGE=6, Z=7, PAD=8, MAXLEN=9, ORIENT=10, NWIN=11, SAMPLE=12,
         WIN=13, ARGMIN=14, MAXSSD=15, UNIQUE=16, DEN=17, CLAMP_HI=18, CLAMP_LO=19, AXIS=20, DOBS=21, INIT=22,
         CHI2=23, VALDROP=24, BLLIMIT=25, RUNBEST=26, RUN2=27, R_HASDEPTH=40, R_NVAL=41, R_COMPAT=42,
         R_SUPPORT=43, R_FILL=44, P_Z=60, P_RX=61, P_RY=62, P_BOUND=63, P_PHOTO=64)
NAME = {v: k for k, v in D.items()}
# decisions whose outcome follows from the pixel's (or a neighbour's) state rather than a threshold
STATE = {D["INIT"], D["VALDROP"], D["BLLIMIT"], D["R_HASDEPTH"], D["R_SUPPORT"], D["R_FILL"]}
FLOOR = {D["NWIN"], D["P_RX"], D["P_RY"]}  # outcome = floor(q)
REG = {D["R_HASDEPTH"], D["R_NVAL"], D["R_COMPAT"], D["R_SUPPORT"], D["R_FILL"]}


def _by_pixel(rec, stage):
    r = rec[rec["stage"] == stage]
    out = {}
    if len(r) == 0:
        return out
    r = r[np.argsort(r["pixel"], kind="stable")]  # stable: keeps the execution order within a pixel
    starts = np.flatnonzero(np.r_[True, r["pixel"][1:] != r["pixel"][:-1]])
    ends = np.r_[starts[1:], len(r)]
    for a, b in zip(starts, ends):
        out[int(r["pixel"][a])] = r[a:b]
    return out


def first_divergence(tf, td):
    """Index of the first record where the two traces of one pixel branch differently (or None)."""
    n = min(len(tf), len(td))
    key = ("id", "ref", "outcome", "aux")
    for k in range(n):
        if any(tf[k][f] != td[k][f] for f in key):
            return k
    return n if len(tf) != len(td) else None


def _rel(a, b, scale):
    return abs(a - b) / max(scale, 1e-30)


def flags_differ(a, b):
    return (a["validity"] != b["validity"]) | (a["blacklist"] != b["blacklist"])


def state_differs(a, b):
    return flags_differ(a, b) | (a["idepth"] != b["idepth"]) | (a["var"] != b["var"])


class Classifier:
    def __init__(self, seq, params=None, tol=2e-3, propagate=True, params_fp64=None):
        # params_fp64 (tests of the classifier only): another parameter table for the FP64 run
        self.seq, self.params, self.tol, self.propagate = seq, params, tol, propagate
        self.params_d = params_fp64 if params_fp64 is not None else params
        self.h, self.w = seq.h, seq.w
        run = lambda dbl, reg: lsdo.depth_pipeline(seq, params=self.params_d if dbl else params, double=dbl,
                                                   regularize=reg, propagate=propagate and reg)
        self.obs_f, _ = run(False, False)
        self.obs_d, _ = run(True, False)
        (self.upd_f, self.prop_f), (self.upd_d, self.prop_d) = run(False, True), run(True, True)
        self._memo = {}

    def _dilate(self, m, r):
        out = m.copy()
        for dy in range(-r, r + 1):
            for dx in range(-r, r + 1):
                out |= np.roll(np.roll(m, dy, 0), dx, 1)
        return out

    def run(self):
        """(update_disagreements, propagation_disagreements): one dict per disagreeing pixel with
        its explanation and, for threshold straddles, the margins."""
        R = (self.params or lsdo.default_params()).reg_radius
        upd_bad = flags_differ(self.upd_f, self.upd_d)
        prop_bad = flags_differ(self.prop_f, self.prop_d) if self.propagate else np.zeros_like(upd_bad)
        # the pixels whose traces can matter: the disagreeing ones and their regularisation windows,
        # every pixel whose state differs after observe or after the update, every old pixel with a
        # hypothesis (propagation), the new keyframe's disagreeing windows
        obs_diff = state_differs(self.obs_f, self.obs_d)
        upd_diff = state_differs(self.upd_f, self.upd_d)
        mask = np.zeros((4, self.h, self.w), bool)
        mask[0] = self._dilate(upd_bad, R) | obs_diff | upd_diff
        mask[1] = self._dilate(upd_bad, R) | upd_diff
        if self.propagate:
            mask[2] = (self.upd_f["validity"] > 0) | (self.upd_d["validity"] > 0)
            mask[3] = self._dilate(prop_bad, R)
        self.tr_f = lsdo.depth_trace(self.seq, mask, double=False, params=self.params, propagate=self.propagate)
        self.tr_d = lsdo.depth_trace(self.seq, mask, double=True, params=self.params_d, propagate=self.propagate)
        self.st = [(_by_pixel(self.tr_f, s), _by_pixel(self.tr_d, s)) for s in range(4)]
        upd = [self.explain(1, int(i)) for i in np.flatnonzero(upd_bad.ravel())]
        prop = [self.explain_target(int(i)) for i in np.flatnonzero(prop_bad.ravel())] if self.propagate else []
        return upd, prop

    # -- one pixel of one stage ---------------------------------------------------------------------
    def diverged(self, stage, pix):
        """None if the pixel's two traces of this stage agree, else (index, rec_f, rec_d, f, d)."""
        f, d = self.st[stage][0].get(pix), self.st[stage][1].get(pix)
        if f is None and d is None:
            return None
        f = f if f is not None else np.zeros(0, lsdo.DECISION_DTYPE)
        d = d if d is not None else np.zeros(0, lsdo.DECISION_DTYPE)
        k = first_divergence(f, d)
        if k is None:
            return None
        return k, (f[k] if k < len(f) else None), (d[k] if k < len(d) else None), f, d

    def straddle(self, rf, rd):
        """(distance of the float quantity to the threshold, float vs FP64 quantity), relative."""
        q_f, q_d, thr = float(rf["q"]), float(rd["q"]), float(rf["thr"])
        if int(rf["id"]) in FLOOR:
            b = np.floor(max(q_f, q_d))  # the integer the two quantities fall either side of
            return _rel(q_f, b, max(1.0, abs(b))), _rel(q_f, q_d, max(1.0, abs(b)))
        scale = max(abs(thr), abs(q_f), abs(q_d))
        return _rel(q_f, thr, scale), _rel(q_f, q_d, scale)

    def explain(self, stage, pix):
        key = (stage, pix)
        if key not in self._memo:
            self._memo[key] = {"explained": False, "why": "cycle"}
            res = self._explain(stage, pix)
            res.update(pixel=pix, stage=stage)
            self._memo[key] = res
        return self._memo[key]

    def _explain(self, stage, pix):
        dv = self.diverged(stage, pix)
        if dv is None:
            # this stage decided alike: the difference comes from an earlier stage
            if stage == 1:
                return self.explain(0, pix)
            if stage == 3:
                return self.explain_target(pix, from_reg=True)
            return {"explained": False, "why": "no divergence found"}
        k, rf, rd, f, _ = dv
        if rf is None or rd is None:
            return {"explained": False, "why": "one trace ended early", "record": k}
        did = int(rf["id"])
        name = NAME.get(did, str(did))
        if stage in (1, 3) and did in REG:
            # a decision over the regularisation window: the pixel's own or a neighbour's state
            others = [pix] + ([int(rf["aux"])] if did in (D["R_NVAL"], D["R_COMPAT"]) else [])
            for o in others:
                if stage == 1 and self.diverged(0, o) is not None:
                    sub = self.explain(0, o)
                    if sub["explained"]:
                        return {"explained": True, "why": f"{name}: state of pixel {o} from observe", "via": sub}
                if stage == 3 and self._target_state_differs(o):
                    sub = self.explain_target(o, from_reg=True)
                    if sub["explained"]:
                        return {"explained": True, "why": f"{name}: state of pixel {o} from propagation", "via": sub}
        if did in STATE:
            return {"explained": False, "why": f"state decision {name} without a diverging input"}
        if did == D["ARGMIN"]:
            sf, sd = int(rf["outcome"]), int(rd["outcome"])
            wins = {int(r["outcome"]): float(r["q"]) for r in f if r["id"] == D["WIN"] and r["ref"] == rf["ref"]}
            if sf in wins and sd in wins and np.isfinite(wins[sf]) and np.isfinite(wins[sd]):
                m = _rel(wins[sf], wins[sd], max(abs(wins[sf]), abs(wins[sd])))
                return {"explained": m <= self.tol, "why": "ARGMIN near-tie of two SSD windows", "margin": m,
                        "ref": int(rf["ref"])}
            return {"explained": False, "why": "ARGMIN without both windows", "ref": int(rf["ref"])}
        m_thr, m_qq = self.straddle(rf, rd)
        return {"explained": m_thr <= self.tol and m_qq <= self.tol, "why": f"{name} threshold straddle",
                "margin_to_threshold": m_thr, "margin_float_vs_fp64": m_qq, "q_float": float(rf["q"]),
                "q_fp64": float(rd["q"]), "threshold": float(rf["thr"]), "ref": int(rf["ref"])}

    # -- propagation ------------------------------------------------------------------------------
    def _warps(self, run):
        """Per old pixel that lands: (target index, float z key) from the stage-2 trace of one run."""
        if not hasattr(self, "_wcache"):
            self._wcache = {}
        if run not in self._wcache:
            tgt, zk = {}, {}
            for o, r in self.st[2][run].items():
                out = {int(i): int(v) for i, v in zip(r["id"], r["outcome"])}
                if out.get(D["P_Z"]) == 1 and out.get(D["P_BOUND"]) == 1 and out.get(D["P_PHOTO"]) == 0:
                    tgt[o] = out[D["P_RY"]] * self.w + out[D["P_RX"]]
                    zk[o] = float(np.float32(r["q"][r["id"] == D["P_Z"]][0]))
            self._wcache[run] = (tgt, zk)
        return self._wcache[run]

    def _target_state_differs(self, t):
        y, x = divmod(t, self.w)
        a, b = self.prop_f, self.prop_d
        return bool(a["validity"][y, x] != b["validity"][y, x] or a["idepth"][y, x] != b["idepth"][y, x] or
                    a["var"][y, x] != b["var"][y, x])

    def _source_differs(self, o):
        y, x = divmod(o, self.w)
        return bool(self.upd_f["idepth"][y, x] != self.upd_d["idepth"][y, x] or
                    self.upd_f["validity"][y, x] != self.upd_d["validity"][y, x])

    def explain_source(self, o):
        """Why old pixel o's hypothesis differs after the update (observe + regularisation)."""
        if self.diverged(1, o) is not None:
            return self.explain(1, o)
        if self.diverged(0, o) is not None:
            return self.explain(0, o)
        return {"explained": False, "why": "source hypothesis differs without a diverging decision", "pixel": o}

    def explain_target(self, t, from_reg=False):
        key = ("t", t, from_reg)
        if key not in self._memo:
            self._memo[key] = {"explained": False, "why": "cycle"}
            res = self._explain_target(t, from_reg)
            res.update(pixel=t, stage=2 if from_reg else 3)
            self._memo[key] = res
        return self._memo[key]

    def _explain_target(self, t, from_reg):
        if not from_reg and self.diverged(3, t) is not None:
            sub = self.explain(3, t)  # the new keyframe's regularisation decided differently
            if sub["explained"]:
                return sub
        tf, zf = self._warps(0)
        td, zd = self._warps(1)
        cands = sorted({o for o, x in tf.items() if x == t} | {o for o, x in td.items() if x == t})
        if not cands:
            return {"explained": False, "why": "no source pixel in either run"}
        for o in cands:  # a source whose warp decisions diverged
            dv = self.diverged(2, o)
            if dv is None:
                continue
            _, rf, rd, _, _ = dv
            if rf is not None and rd is not None:
                m_thr, m_qq = self.straddle(rf, rd)
                if m_thr <= self.tol and m_qq <= self.tol:
                    return {"explained": True, "why": f"source {o}: {NAME[int(rf['id'])]} threshold straddle",
                            "margin_to_threshold": m_thr, "margin_float_vs_fp64": m_qq}
            if self._source_differs(o):
                sub = self.explain_source(o)
                if sub["explained"]:
                    return {"explained": True, "why": f"source {o}: hypothesis from the update", "via": sub}
        for o in cands:  # a source whose hypothesis or validity differs after the update
            if self._source_differs(o):
                sub = self.explain_source(o)
                if sub["explained"]:
                    return {"explained": True, "why": f"source {o}: state from the update", "via": sub}
        cf = [o for o in cands if tf.get(o) == t]
        cd = [o for o in cands if td.get(o) == t]
        if cf and cd:  # same candidates, another winner: a near-tie of their depths
            wf = min(cf, key=lambda o: (zf[o], o))
            wd = min(cd, key=lambda o: (zd[o], o))
            if wf != wd and wd in zf:
                m = _rel(zf[wf], zf[wd], abs(zf[wf]))
                return {"explained": m <= self.tol, "why": "z-buffer near-tie", "margin": m}
        return {"explained": False, "why": "propagation: no diverging decision found", "candidates": cands}


def classify(seq, params=None, tol=2e-3, propagate=True, params_fp64=None):
    """Runs the float and FP64 oracles on `seq` and explains every flag disagreement."""
    c = Classifier(seq, params, tol, propagate, params_fp64)
    upd, prop = c.run()
    return c, upd, prop


def worst_margin(results):
    """Largest relative margin among the explanations (threshold or float-vs-FP64)."""
    m = 0.0
    for r in results:
        while "via" in r:
            r = r["via"]
        for k in ("margin", "margin_to_threshold", "margin_float_vs_fp64"):
            if k in r:
                m = max(m, float(r[k]))
    return m
