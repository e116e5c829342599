"""Extended-precision (numpy longdouble) evaluation of logL and the branch
gradient, test infrastructure: it measures how far any FP64 evaluation (the
oracle's, the GPU's) is from a more precise one on the same inputs, which is
what the FP64 gradient tolerance has to allow for."""
import numpy as np

from mcphylo_gb300.tree import nodes_by_num, post_order

LD = np.longdouble
def ext_grad(inst):
    """(ll, grad) in longdouble; pre-order partials rescaled by their maximum."""
    K=inst.K; C=len(inst.rates); S=inst.S
    U=inst.U.astype(LD); D=inst.D.astype(LD); Ui=inst.Uinv.astype(LD); mu=LD(inst.mu); r=inst.rates.astype(LD)
    by=nodes_by_num(inst.tree); N=len(by)
    blen=inst.blen.astype(LD)
    P={}; dP={}
    for n in by[:-1]:
        for c in range(C):
            e=np.exp(mu*blen[n.num-1]*D*r[c])
            P[n.num,c]=(U*e[None,:])@Ui
            dP[n.num,c]=(U*(D*r[c]*mu*e)[None,:])@Ui
    x=inst.tensor()
    L={}; Dn={}
    ll=LD(0)
    for n in post_order(inst.tree):
        if not n.children:
            L[n.num]=[x[:,:,n.num-1].astype(LD) for c in range(C)]  # (K,S)
            continue
        L[n.num]=[]
        for c in range(C):
            prod=np.ones((K,S),dtype=LD)
            for ch in n.children:
                d=P[ch.num,c]@L[ch.num][c]; Dn[ch.num,c]=d; prod*=d
            L[n.num].append(prod)
    root=post_order(inst.tree)[-1]
    pi=inst.pi.astype(LD)
    for c in range(C):
        ll+=np.sum(np.log(pi@L[root.num][c]))
    # pre-order
    pre={}
    g=np.zeros(N-1,dtype=LD)
    order=list(reversed(post_order(inst.tree)))
    for c in range(C):
        pre[root.num,c]=np.tile(pi[:,None],(1,S))
    for n in order[1:]:
        m=n.mother
        for c in range(C):
            pt=pre[m.num,c].copy()
            for s in m.children:
                if s is not n: pt*=Dn[s.num,c]
            num=np.sum(pt*(dP[n.num,c]@L[n.num][c]),axis=0)
            den=np.sum(pt*(P[n.num,c]@L[n.num][c]),axis=0)
            g[n.num-1]+=np.sum(num/den)
            pb=P[n.num,c].T@pt
            pb/=pb.max(axis=0,keepdims=True)
            pre[n.num,c]=pb
    return ll,g

