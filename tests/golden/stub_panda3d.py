"""Stand-ins for Panda3D, TorchRL and tensordict so that the reference's
unmodified Python scene code can be imported and run without a graphics stack.

TEST INFRASTRUCTURE ONLY: used by ``make_golden.py`` (in this directory) to
record the exact buffers the reference would upload to OpenGL -- per-instance
model matrices (``matbuf``), colours (``colbuf``), per-scene view-projection
matrices (``viewbuf``), tile rectangles (``tilebuf``), shader uniforms, and the
vertex positions after model scale / pivot baking.  Nothing is drawn.

Modelled Panda3D behaviour (only what the reference's scene code touches):
``NodePath`` local transforms (scale, then rotation, then translation),
``flattenStrong`` (bakes this node's and its descendants' transforms into their
vertices), ``getTightBounds``, ``wrtReparentTo`` / ``setPos(other, p)``,
``Texture.set_ram_image`` (records the bytes), ``setShaderInput`` (records the
value), ``loadPrcFileData`` (``win-size``), and ``loader.loadModel("models/box")``,
which returns Panda3D's bundled unit box (``[0,1]^3``, one quad per face) as
24 vertices.
"""
from __future__ import annotations

import math
import sys
import types

import numpy as np

_PRC = {"win-size": (800, 600)}


def load_prc_file_data(name, data):
    for line in str(data).splitlines():
        parts = line.split()
        if len(parts) == 3 and parts[0] == "win-size":
            _PRC["win-size"] = (int(parts[1]), int(parts[2]))


def _panda_hpr(h, p, r):
    h, p, r = (math.radians(float(a)) for a in (h, p, r))
    ch, sh, cp, sp, cr, sr = math.cos(h), math.sin(h), math.cos(p), math.sin(p), math.cos(r), math.sin(r)
    rz = np.array([[ch, -sh, 0], [sh, ch, 0], [0, 0, 1]])
    rx = np.array([[1, 0, 0], [0, cp, -sp], [0, sp, cp]])
    ry = np.array([[cr, 0, sr], [0, 1, 0], [-sr, 0, cr]])
    return rz @ rx @ ry


class LPoint3:
    def __init__(self, x=0.0, y=0.0, z=0.0):
        self.x, self.y, self.z = float(x), float(y), float(z)

    def __getitem__(self, i):
        return (self.x, self.y, self.z)[i]

    def __neg__(self):
        return LPoint3(-self.x, -self.y, -self.z)

    def __bool__(self):
        return True


Vec3 = LPoint3


class _Node:
    def __init__(self, owner):
        self.owner = owner

    def setBounds(self, b):
        pass

    def setFinal(self, f):
        pass

    def getLens(self):
        return None

    def setLens(self, lens):
        pass


class NodePath:
    def __init__(self, name="node", verts=None):
        self.name = name
        self.parent = None
        self.children = []
        self.verts = None if verts is None else np.asarray(verts, np.float64).copy()
        self.scale = np.ones(3)
        self.hpr = np.zeros(3)
        self.pos = np.zeros(3)
        self.shader_inputs = {}
        self.instance_count = None
        self._node = _Node(self)

    # transforms ------------------------------------------------------------
    def local_matrix(self):
        m = np.eye(4)
        m[:3, :3] = _panda_hpr(*self.hpr) @ np.diag(self.scale)
        m[:3, 3] = self.pos
        return m

    def world_matrix(self):
        m = self.local_matrix()
        p = self.parent
        while p is not None:
            m = p.local_matrix() @ m
            p = p.parent
        return m

    def setScale(self, *s):
        self.scale = np.array(s if len(s) == 3 else (s[0],) * 3, float)

    def setHpr(self, *a):
        self.hpr = np.array(a, float)

    def setPos(self, *args):
        if len(args) == 2 and isinstance(args[0], NodePath):
            other, p = args
            want_world = other.world_matrix() @ np.array([p[0], p[1], p[2], 1.0])
            parent_w = self.parent.world_matrix() if self.parent is not None else np.eye(4)
            self.pos = (np.linalg.inv(parent_w) @ want_world)[:3]
        else:
            p = args[0] if len(args) == 1 else args
            self.pos = np.array([p[0], p[1], p[2]], float)

    def getTightBounds(self, other=None):
        pts = []
        base_inv = np.linalg.inv(other.world_matrix()) if other is not None else np.eye(4)

        def walk(n):
            if n.verts is not None and len(n.verts):
                m = base_inv @ n.world_matrix()
                v = np.c_[n.verts, np.ones(len(n.verts))] @ m.T
                pts.append(v[:, :3])
            for c in n.children:
                walk(c)
        walk(self)
        if not pts:
            return None
        allp = np.concatenate(pts)
        lo, hi = allp.min(axis=0), allp.max(axis=0)
        return LPoint3(*lo), LPoint3(*hi)

    def flattenStrong(self):
        def bake(n, acc):
            m = acc @ n.local_matrix()
            if n.verts is not None and len(n.verts):
                n.verts = (np.c_[n.verts, np.ones(len(n.verts))] @ m.T)[:, :3]
            n.scale, n.hpr, n.pos = np.ones(3), np.zeros(3), np.zeros(3)
            for c in n.children:
                bake(c, m)
        bake(self, np.eye(4))

    flattenLight = flattenStrong
    flattenMedium = flattenStrong

    # hierarchy -------------------------------------------------------------
    def reparentTo(self, parent):
        if self.parent is not None:
            self.parent.children.remove(self)
        self.parent = parent
        parent.children.append(self)

    def wrtReparentTo(self, parent):
        w = self.world_matrix()
        self.reparentTo(parent)
        local = np.linalg.inv(parent.world_matrix()) @ w
        # decompose (the reference only moves nodes with pure translations here)
        self.pos = local[:3, 3].copy()
        sc = np.linalg.norm(local[:3, :3], axis=0)
        self.scale = sc
        self.hpr = np.zeros(3)

    def attachNewNode(self, name):
        n = NodePath(name if isinstance(name, str) else "node")
        n.reparentTo(self)
        return n

    def getParent(self):
        return self.parent

    def removeNode(self):
        if self.parent is not None:
            self.parent.children.remove(self)
            self.parent = None

    def clearModelNodes(self):
        pass

    def set_instance_count(self, n):
        self.instance_count = int(n)

    def setShader(self, s):
        pass

    def setShaderInput(self, name, value):
        self.shader_inputs[name] = value

    def setTexture(self, t):
        pass

    def node(self):
        return self._node

    def getPos(self, other=None):
        return LPoint3(*self.pos)


def _unit_box():
    faces = [((1, 0, 0), (0, 1, 0), (0, 0, 1)), ((0, 1, 0), (0, -1, 0), (0, 0, 1)),
             ((1, 1, 0), (-1, 0, 0), (0, 0, 1)), ((0, 0, 0), (1, 0, 0), (0, 0, 1)),
             ((0, 0, 1), (1, 0, 0), (0, 1, 0)), ((0, 1, 0), (1, 0, 0), (0, -1, 0))]
    v = []
    for o, u, w in faces:
        o, u, w = np.array(o, float), np.array(u, float), np.array(w, float)
        v += [o, o + u, o + u + w, o + w]
    return np.array(v)


class Loader:
    def loadModel(self, path):
        name = str(path)
        if name.endswith("box") or name.endswith("box.egg"):
            return NodePath("box", _unit_box())
        raise FileNotFoundError(f"stub loader has no model {path!r}")

    def loadTexture(self, path):
        return Texture(str(path))


class Texture:
    T_float = 0
    F_rgba32 = 0
    CMOff = 0

    def __init__(self, name=""):
        self.name = name
        self.ram = None
        self.texels = 0

    def setupBufferTexture(self, texels, comp, fmt, usage):
        self.texels = int(texels)

    def set_keep_ram_image(self, keep):
        pass

    setKeepRamImage = set_keep_ram_image

    def set_ram_image(self, data):
        self.ram = bytes(data)

    def setCompression(self, c):
        pass

    def array(self, shape):
        return np.frombuffer(self.ram, dtype=np.float32).reshape(shape).copy()


class _Gsg:
    def getDriverRenderer(self):
        return "stub"


class _Buffer:
    def __init__(self, w, h):
        self.w, self.h = w, h
        self.tex = Texture("buffer")

    def setClearColor(self, c):
        self.clear = c

    def setClearColorActive(self, a):
        pass

    def getTexture(self):
        return self.tex

    def getXSize(self):
        return self.w

    def getYSize(self):
        return self.h


class _Win:
    def __init__(self, w, h):
        self.w, self.h = w, h
        self.pipe = types.SimpleNamespace(getType=lambda: types.SimpleNamespace(getName=lambda: "stub"))

    def getXSize(self):
        return self.w

    def getYSize(self):
        return self.h

    def getGsg(self):
        return _Gsg()

    def getDisplayRegions(self):
        return []

    def setActive(self, a):
        pass

    def makeTextureBuffer(self, name, w, h):
        return _Buffer(w, h)


class _TaskMgr:
    def add(self, fn, name=None):
        pass

    def step(self):
        pass

    def doMethodLater(self, delay, fn, name=None):
        pass


class ShowBase:
    def __init__(self, *a, **k):
        w, h = _PRC["win-size"]
        self.win = _Win(w, h)
        self.render = NodePath("render")
        self.loader = Loader()
        self.taskMgr = _TaskMgr()
        self.cam = NodePath("cam")
        self.graphicsEngine = types.SimpleNamespace(extractTextureData=lambda *a: None)
        self.mouseWatcherNode = types.SimpleNamespace(hasMouse=lambda: False)
        self.a2dTopLeft = NodePath("a2d")

    def disableMouse(self):
        pass

    def setBackgroundColor(self, *c):
        self._stub_bg = c

    def makeCamera(self, buf):
        return NodePath("cam2")

    def accept(self, *a, **k):
        pass


class _Task:
    cont = 1
    done = 0


def install() -> None:
    """Register the stand-in modules in ``sys.modules``."""
    core = types.ModuleType("panda3d.core")
    core.loadPrcFileData = load_prc_file_data
    core.Texture = Texture
    core.NodePath = NodePath
    core.OmniBoundingVolume = lambda *a: object()
    core.Shader = types.SimpleNamespace(make=lambda *a: object(), SL_GLSL=0)
    core.GeomEnums = types.SimpleNamespace(UH_dynamic=0)
    core.MouseButton = types.SimpleNamespace(one=lambda: 0)
    core.TextNode = types.SimpleNamespace(ALeft=0)
    core.LPoint3 = LPoint3
    core.Vec3 = Vec3
    panda3d = types.ModuleType("panda3d")
    panda3d.core = core
    direct = types.ModuleType("direct")
    sb = types.ModuleType("direct.showbase")
    sbm = types.ModuleType("direct.showbase.ShowBase")
    sbm.ShowBase = ShowBase
    sbg = types.ModuleType("direct.showbase.ShowBaseGlobal")
    sbg.globalClock = types.SimpleNamespace(getRealTime=lambda: 0.0, getAverageFrameRate=lambda: 0.0)
    task = types.ModuleType("direct.task")
    task.Task = _Task
    gui = types.ModuleType("direct.gui")
    ost = types.ModuleType("direct.gui.OnscreenText")
    ost.OnscreenText = lambda *a, **k: types.SimpleNamespace(setText=lambda t: None)
    td = types.ModuleType("tensordict")

    class TensorDict(dict):
        def __init__(self, fields=None, batch_size=None, **k):
            super().__init__(fields or {})
            self.batch_size = batch_size
    td.TensorDict = TensorDict
    trl = types.ModuleType("torchrl")
    envs = types.ModuleType("torchrl.envs")

    class EnvBase:
        def __init__(self, device=None, batch_size=None, **k):
            self.device, self.batch_size = device, batch_size

        def set_seed(self, seed=None, static_seed=False):
            # TorchRL's EnvBase.set_seed hands the seed to the subclass hook
            self._set_seed(seed)
            return seed
    envs.EnvBase = EnvBase
    envs.ParallelEnv = object
    data = types.ModuleType("torchrl.data")
    specs = types.ModuleType("torchrl.data.tensor_specs")
    for nm in ("Composite", "Unbounded", "Categorical", "Bounded"):
        setattr(specs, nm, lambda *a, **k: types.SimpleNamespace(**k))
    mods = {
        "panda3d": panda3d, "panda3d.core": core, "direct": direct, "direct.showbase": sb,
        "direct.showbase.ShowBase": sbm, "direct.showbase.ShowBaseGlobal": sbg, "direct.task": task,
        "direct.gui": gui, "direct.gui.OnscreenText": ost, "tensordict": td, "torchrl": trl,
        "torchrl.envs": envs, "torchrl.data": data, "torchrl.data.tensor_specs": specs,
    }
    sys.modules.update(mods)
