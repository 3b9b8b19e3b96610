"""Host-memory placement for host-buffer SpMM.

Pinned host buffers are placed by first touch: the memory node of the CPU
that writes a page first holds it.  On machines with several CPU sockets or
memory nodes, a buffer on a node far from the GPU crosses the inter-socket
link on every copy.  ``bind_to_device_cpus`` restricts the calling process
to the CPUs the GPU's PCI function lists as local (sysfs ``local_cpulist``),
so buffers allocated and filled afterwards land next to the GPU.  Where the
sysfs entry is missing it does nothing and says so.
"""
from __future__ import annotations

import os

import torch


def _parse_cpulist(text: str) -> list[int]:
    cpus: list[int] = []
    for part in text.strip().split(","):
        if not part:
            continue
        if "-" in part:
            a, b = part.split("-", 1)
            cpus.extend(range(int(a), int(b) + 1))
        else:
            cpus.append(int(part))
    return cpus


def device_pci_path(device) -> str | None:
    """sysfs directory of the device's PCI function, or None."""
    dev = torch.device(device)
    idx = dev.index if dev.index is not None else torch.cuda.current_device()
    props = torch.cuda.get_device_properties(idx)
    dom = getattr(props, "pci_domain_id", None)
    bus = getattr(props, "pci_bus_id", None)
    slot = getattr(props, "pci_device_id", None)
    if bus is None or slot is None:
        return None
    path = f"/sys/bus/pci/devices/{int(dom or 0):04x}:{int(bus):02x}:{int(slot):02x}.0"
    return path if os.path.isdir(path) else None


def bind_to_device_cpus(device) -> dict:
    """Restrict this process to the CPUs local to ``device``; returns what was
    found and done (``bound`` False when there was nothing to bind to)."""
    info: dict = {"bound": False}
    path = device_pci_path(device)
    if path is None:
        info["reason"] = "no sysfs PCI entry for the device"
        return info
    try:
        with open(os.path.join(path, "numa_node")) as f:
            info["numa_node"] = int(f.read().strip())
    except OSError:
        pass
    try:
        with open(os.path.join(path, "local_cpulist")) as f:
            local = _parse_cpulist(f.read())
    except OSError:
        info["reason"] = "no local_cpulist"
        return info
    allowed = sorted(os.sched_getaffinity(0))
    cpus = sorted(set(local) & set(allowed))
    info["local_cpus"] = len(local)
    info["allowed_cpus"] = len(allowed)
    if not cpus:
        info["reason"] = "none of the device's local CPUs is available to this process"
        return info
    if cpus != allowed:
        os.sched_setaffinity(0, cpus)
    info["bound"] = True
    info["cpus"] = len(cpus)
    info["_previous"] = allowed
    return info


def restore_cpus(info: dict) -> None:
    """Undo ``bind_to_device_cpus`` (buffers already placed stay where they are)."""
    prev = info.pop("_previous", None)
    if prev:
        os.sched_setaffinity(0, prev)
