"""Process-replica parallel environment: the ``ParallelEnv`` behind
``PBREnv.make_parallel_env`` / ``envs.make_parallel`` when TorchRL is not
installed (``pybatchrender/env.py:360-440``, ``envs/__init__.py:127-164`` of
the reference build a TorchRL ``ParallelEnv`` of spawned workers).

Each worker is a spawned process that builds its own env and renderer with
``create_env_fn(**create_env_kwargs[i])`` -- its own CUDA context, on its own
device when the configs name different devices, which is how this renderer
scales over several GPUs (scenes are independent: nothing is exchanged).
The main process sees one env of batch ``[num_workers, *worker_batch]``:

* ``reset()`` / ``step(td)`` / ``td["next"]`` / ``action_spec.rand()`` /
  ``set_seed`` / ``close()``, the slice of TorchRL's ``ParallelEnv`` the
  reference's benchmark uses;
* with ``shared_memory=True`` the per-step tensors live in buffers the main
  process allocates once per key (CPU shared memory, or CUDA memory shared
  with the workers through CUDA IPC when every worker runs on the main
  process's CUDA device): workers read their action slice and write their
  results in place, and only short commands cross the pipes.  With
  ``shared_memory=False`` every step's tensors are sent through the pipes.

Errors in a worker are re-raised in the main process as ``RuntimeError``
with the worker's traceback; a worker that dies is reported the same way.
"""
from __future__ import annotations

import traceback

import torch
import torch.multiprocessing as tmp

from .env import TensorDict, _SpecLite


def _flatten(td, prefix=()) -> dict:
    out = {}
    for k in list(td.keys()):
        v = td[k]
        if torch.is_tensor(v):
            out[prefix + (k,)] = v
        elif hasattr(v, "keys"):
            out.update(_flatten(v, prefix + (k,)))
    return out


def _unflatten(flat: dict, batch_size) -> "TensorDict":
    td = TensorDict({}, batch_size=batch_size)
    for key, v in flat.items():
        cur = td
        for part in key[:-1]:
            if part not in cur.keys():
                cur[part] = TensorDict({}, batch_size=batch_size)
            cur = cur[part]
        cur[key[-1]] = v
    return td


def _spec_meta(spec):
    if spec is None:
        return None
    return {"shape": tuple(spec.shape), "dtype": spec.dtype, "n": getattr(spec, "n", None),
            "low": getattr(spec, "low", None), "high": getattr(spec, "high", None)}


def _sync_device(device: torch.device) -> None:
    if device.type == "cuda":
        torch.cuda.synchronize(device)


def _worker(conn, create_env_fn, kwargs) -> None:  # pragma: no cover - runs in the spawned process
    """Serve commands for one env until ``close``."""
    try:
        env = create_env_fn(**kwargs)
        dev = torch.device(env.device)
        if dev.type == "cuda" and dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        bufs = {"reset": None, "step": None, "in": None}
        conn.send(("ready", {"batch_size": tuple(env.batch_size), "device": str(dev),
                             "action_spec": _spec_meta(getattr(env, "action_spec", None))}))
    except BaseException:
        conn.send(("err", traceback.format_exc()))
        return
    while True:
        try:
            cmd, arg = conn.recv()
        except EOFError:
            return
        try:
            if cmd == "close":
                close = getattr(env, "close", None)
                if callable(close):
                    close()
                conn.send(("ok", None))
                return
            if cmd == "bufs":  # buffers (slices) to read or write in place from now on
                name, views = arg
                bufs[name] = views
                conn.send(("ok", None))
            elif cmd == "seed":
                env.set_seed(int(arg))
                conn.send(("ok", None))
            elif cmd in ("reset", "step"):
                if cmd == "reset":
                    out = _flatten(env.reset())
                else:
                    inp = arg if arg is not None else bufs["in"]
                    td = _unflatten({k: v.to(dev) for k, v in inp.items()}, env.batch_size)
                    res = env.step(td)
                    out = _flatten(res["next"] if "next" in res.keys() else res)
                if bufs[cmd] is not None and set(bufs[cmd]) == set(out):
                    for k, v in out.items():
                        bufs[cmd][k].copy_(v)
                    _sync_device(bufs[cmd][next(iter(bufs[cmd]))].device)
                    conn.send(("ok", None))
                else:
                    conn.send(("data", {k: v.detach().cpu() for k, v in out.items()}))
            else:
                conn.send(("err", f"unknown command {cmd!r}"))
        except BaseException:
            conn.send(("err", traceback.format_exc()))


class ParallelEnvLite:
    """``num_workers`` env replicas in spawned processes, seen as one env of
    batch ``[num_workers, *worker_batch]`` (see the module docstring)."""

    def __init__(self, num_workers: int, create_env_fn, create_env_kwargs: list[dict] | dict | None = None,
                 mp_start_method: str = "spawn", shared_memory: bool = True):
        self.num_workers = int(num_workers)
        if self.num_workers < 1:
            raise ValueError("num_workers must be >= 1")
        if create_env_kwargs is None:
            create_env_kwargs = {}
        if isinstance(create_env_kwargs, dict):
            create_env_kwargs = [dict(create_env_kwargs) for _ in range(self.num_workers)]
        if len(create_env_kwargs) != self.num_workers:
            raise ValueError("create_env_kwargs needs one entry per worker")
        self.shared_memory = bool(shared_memory)
        ctx = tmp.get_context(mp_start_method)
        self._conns, self._procs = [], []
        self._closed = False
        for kw in create_env_kwargs:
            parent, child = ctx.Pipe()
            p = ctx.Process(target=_worker, args=(child, create_env_fn, kw), daemon=True)
            p.start()
            child.close()
            self._conns.append(parent)
            self._procs.append(p)
        metas = [self._recv(i) for i in range(self.num_workers)]
        inner = metas[0]["batch_size"]
        if any(m["batch_size"] != inner for m in metas):
            self.close()
            raise ValueError("every worker env must have the same batch size")
        self.worker_devices = [torch.device(m["device"]) for m in metas]
        self.device = self.worker_devices[0]
        self.batch_size = torch.Size([self.num_workers, *inner])
        # shared buffers on the workers' CUDA device only when all of them use this process's device
        same = all(d == self.device for d in self.worker_devices)
        self._buf_device = self.device if (self.device.type == "cuda" and same) else torch.device("cpu")
        a = metas[0]["action_spec"]
        self.action_spec = None
        if a is not None:
            shape = torch.Size([self.num_workers, *a["shape"]])
            self.action_spec = _SpecLite(shape, a["dtype"], self.device, n=a["n"], low=a["low"], high=a["high"])
        self._out = {"reset": None, "step": None}
        self._in = None

    # -------------------------------------------------------------- plumbing
    def _recv(self, i):
        try:
            kind, payload = self._conns[i].recv()
        except EOFError:
            raise RuntimeError(f"worker {i} exited (exit code {self._procs[i].exitcode})") from None
        if kind == "err":
            raise RuntimeError(f"worker {i} failed:\n{payload}")
        return payload

    def _broadcast(self, cmd, args):
        for i, conn in enumerate(self._conns):
            conn.send((cmd, args[i] if isinstance(args, list) else args))
        return [self._recv(i) for i in range(self.num_workers)]

    def _alloc(self, like: dict) -> dict:
        bufs = {}
        for k, v in like.items():
            t = torch.empty((self.num_workers, *v.shape), dtype=v.dtype, device=self._buf_device)
            if t.device.type == "cpu":
                t.share_memory_()
            bufs[k] = t
        return bufs

    def _gather(self, name: str, replies) -> dict:
        """Stacked results of a reset or step: the shared buffers, or the
        tensors the workers sent (and, the first time, the buffers for the next call)."""
        if all(r is None for r in replies):
            bufs = self._out[name]
        else:
            flat = {k: torch.stack([r[k] for r in replies]) for k in replies[0]}
            if not self.shared_memory:
                return {k: v.to(self.device) for k, v in flat.items()}
            bufs = self._alloc({k: v[0] for k, v in flat.items()})
            for k, v in flat.items():
                bufs[k].copy_(v)
            self._out[name] = bufs
            self._broadcast("bufs", [(name, {k: v[i] for k, v in bufs.items()}) for i in range(self.num_workers)])
        # copies: the buffers are overwritten by the next call
        return {k: v.to(self.device, copy=True) for k, v in bufs.items()}

    # ------------------------------------------------------------------- API
    def reset(self, tensordict=None):
        replies = self._broadcast("reset", None)
        return _unflatten(self._gather("reset", replies), self.batch_size)

    def step(self, tensordict):
        flat = {k: v for k, v in _flatten(tensordict).items() if k[0] != "next"}
        if self.shared_memory:
            if self._in is None or set(self._in) != set(flat) or any(
                    self._in[k].shape[1:] != v.shape[1:] or self._in[k].dtype != v.dtype for k, v in flat.items()):
                self._in = self._alloc({k: v[0] for k, v in flat.items()})
                self._broadcast("bufs", [("in", {k: v[i] for k, v in self._in.items()})
                                         for i in range(self.num_workers)])
            for k, v in flat.items():
                self._in[k].copy_(v)
            _sync_device(self._buf_device)
            replies = self._broadcast("step", None)
        else:
            replies = self._broadcast("step", [{k: v[i].detach().cpu() for k, v in flat.items()}
                                               for i in range(self.num_workers)])
        tensordict["next"] = _unflatten(self._gather("step", replies), self.batch_size)
        return tensordict

    def rand_action(self, tensordict=None):
        td = tensordict if tensordict is not None else TensorDict({}, batch_size=self.batch_size)
        td["action"] = self.action_spec.rand()
        return td

    def set_seed(self, seed: int, static_seed: bool = False):
        self._broadcast("seed", [int(seed) + i for i in range(self.num_workers)])
        return seed

    def close(self) -> None:
        if self._closed:
            return
        self._closed = True
        for i, conn in enumerate(self._conns):
            try:
                if self._procs[i].is_alive():
                    conn.send(("close", None))
                    conn.recv()
            except (EOFError, BrokenPipeError, OSError):
                pass
        for p in self._procs:
            p.join(timeout=30)
            if p.is_alive():
                p.terminate()
                p.join(timeout=5)
        for conn in self._conns:
            conn.close()

    @property
    def is_closed(self) -> bool:
        return self._closed

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
