"""Multi-GPU serving is replicas: one server per device and a host-side
dispatcher.  Checked on CPU with fake servers: requests go to the replica
with the most uncommitted budget, results come back under the dispatcher's
tickets with their device, and the load is released at completion."""
from mphimplicit_gb300.serving import ReplicaDispatcher


class FakeServer:
    def __init__(self, device):
        self.device = device
        self.next = 1
        self.pending = []
        self.done = []
        self.closed = False

    def submit(self, params, parts, dim, steps, precision=0, fields=()):
        t = self.next
        self.next += 1
        self.pending.append(t)
        return t

    def finish_all(self):
        self.done, self.pending = self.pending, []

    def poll(self, wait_ms=0):
        out = [{"ticket": t, "status": 0, "steps": 1} for t in self.done]
        self.done = []
        return out

    def close(self):
        self.closed = True


def test_dispatch_balances_by_uncommitted_budget():
    d = ReplicaDispatcher([0, 1, 2], budget_bytes=100, server_factory=FakeServer)
    sizes = [50, 10, 10, 30, 20, 5]
    tickets = [d.submit(None, None, 2, 1, footprint_bytes=s) for s in sizes]
    # 50 -> r0; 10 -> r1; 10 -> r2; 30 -> r1 (tie with r2, lower index); 20 -> r2; 5 -> r2
    assert [d.route[t][0] for t in tickets] == [0, 1, 2, 1, 2, 2]
    assert d.queued == [50, 40, 35]
    for s in d.servers:
        s.finish_all()
    res = d.poll()
    assert sorted(r["ticket"] for r in res) == tickets
    assert {r["ticket"]: r["device"] for r in res}[tickets[0]] == 0
    assert d.queued == [0, 0, 0] and d.outstanding() == 0
    d.close()
    assert all(s.closed for s in d.servers)
