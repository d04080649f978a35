% Grid, reference data and device upload (advection/preprocessProblem.m:48-112).  The velocity is
% projected once (it is time-independent in the advection test cases) and uploaded with the mesh.
function problemData = preprocessProblem(problemData)
[~, ~, ~, subStepList] = getStepLists();   % sub-step handles, as advection/preprocessProblem.m:50-51
problemData.subStepHandles = getStepHandles(problemData.problemName, subStepList);
problemData.g = problemData.generateGridData(problemData.hmax);
g = problemData.g;
problemData.K = g.numT;
problemData.N = nchoosek(problemData.p + 2, problemData.p);
problemData.tau = problemData.tEnd / problemData.numSteps;
g.markE0Tint  = problemData.generateMarkE0Tint(g);
g.markE0TbdrN = problemData.generateMarkE0TbdrN(g);
g.markE0TbdrD = problemData.generateMarkE0TbdrD(g);
problemData.g = g;
problemData.basesOnQuad = computeBasesOnQuad(problemData.N, struct);
problemData.hatM = integrateRefElemPhiPhi(problemData.N, problemData.basesOnQuad);
limTypes = struct('linear', 0, 'hierarch_vert', 1, 'strict', 2);
precs = struct('fp64', 0, 'fp32', 1, 'df32', 2);   % DGADV_FP64, DGADV_FP32, DGADV_DF32
prec = precs.(problemData.precision);
opts = [problemData.p, problemData.ordRK, prec, problemData.isSlopeLim, ...
        limTypes.(problemData.typeSlopeLim), problemData.device, problemData.gpuFlags];
problemData.gpu = dgadv_mex('create', g.coordV, g.V0T, g.idE0T, g.markE0TbdrD, g.markE0TbdrN, opts);
u1Disc = projectFuncCont2DataDisc(g, @(x1,x2) problemData.u1Cont(0,x1,x2), 2*problemData.p, problemData.hatM, problemData.basesOnQuad);
u2Disc = projectFuncCont2DataDisc(g, @(x1,x2) problemData.u2Cont(0,x1,x2), 2*problemData.p, problemData.hatM, problemData.basesOnQuad);
vN = computeFuncContNuOnQuadEdge(g, @(x1,x2) problemData.u1Cont(0,x1,x2), @(x1,x2) problemData.u2Cont(0,x1,x2), 2*problemData.p+1);
dgadv_mex('set_velocity', problemData.gpu, u1Disc, u2Disc, vN);
end % function
