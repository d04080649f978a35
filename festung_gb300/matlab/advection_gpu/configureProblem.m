% Configuration of the advection_gpu problem on triangles.  The reference's own test cases
% ('solid_body', 'transient') are configured by the reference's advection/configureProblem.m.
% The cases of the benchmark workloads ('gauss_slot', 'ensemble', 'adjoint') are defined here:
% that file's switch stops with 'Invalid testcase' for any other name
% (advection/configureProblem.m:134-135).  Their defaults are the reference's
% (advection/configureProblem.m:63-87) on triangles, and their closures are those of the Python
% mirror (festung_gb300/testcases.py), with the same signatures as the reference's: c0Cont(x1,x2),
% u1Cont / u2Cont / fCont / cDCont / gNCont (t,x1,x2).
function problemData = configureProblem(problemData)
problemData = setdefault(problemData, 'testcase', 'solid_body');
problemData = setdefault(problemData, 'isQuadri', false);
assert(~problemData.isQuadri, 'advection_gpu runs on triangles only.')
problemData = setdefault(problemData, 'isVisSol', false);
problemData = setdefault(problemData, 'precision', 'fp64');   % 'fp64' | 'fp32' | 'df32'
problemData = setdefault(problemData, 'device', 0);
problemData = setdefault(problemData, 'gpuFlags', 0);
switch problemData.testcase
  case {'solid_body', 'transient'}
    problemData = execin('advection/configureProblem', problemData);
    return
  case {'gauss_slot', 'ensemble', 'adjoint'}
  otherwise
    error('Invalid testcase "%s".', problemData.testcase);
end % switch
if strcmp(problemData.testcase, 'ensemble')   % an instance sets its own mesh level and degree
  problemData = setdefault(problemData, 'ensembleParams', ensembleParams(problemData));
  problemData = setdefault(problemData, 'hmax', 2^-problemData.ensembleParams.level);
  problemData = setdefault(problemData, 'p', problemData.ensembleParams.p);
  problemData = setdefault(problemData, 'meshSeed', problemData.ensembleParams.meshSeed);
end % if
%% Defaults of advection/configureProblem.m:63-87 (triangles).
problemData = setdefault(problemData, 'hmax', 2^-6);
problemData = setdefault(problemData, 'p', 0);
problemData = setdefault(problemData, 'qOrd', 2*problemData.p + 1);
problemData = setdefault(problemData, 'qOrdMax', problemData.qOrd);
problemData = setdefault(problemData, 'ordRK', min(problemData.p+1,3));
problemData = setdefault(problemData, 'numSteps', 100);
problemData = setdefault(problemData, 'tEnd', (problemData.numSteps/(3142*1.5))*2*pi);
problemData = setdefault(problemData, 'isSlopeLim', false);
problemData = setdefault(problemData, 'typeSlopeLim', 'linear');
problemData = setdefault(problemData, 'isVisGrid', false);
problemData = setdefault(problemData, 'outputFrequency', 100);
problemData = setdefault(problemData, 'outputBasename', ['output' filesep 'advection_' problemData.typeSlopeLim]);
problemData = setdefault(problemData, 'outputTypes', { 'vtk' });
assert(problemData.p >= 0 && problemData.p <= 3, 'Polynomial order must be zero to three on the device.')
assert(problemData.ordRK >= 1 && problemData.ordRK <= 3, 'Order of Runge Kutta must be zero to three.')
assert(problemData.hmax > 0, 'Maximum edge length must be positive.')
assert(problemData.numSteps > 0, 'Number of time steps must be positive.')
assert(~problemData.isSlopeLim || problemData.p > 0, 'Slope limiting only available for p > 0.')
problemData.isAnalytical = false;
problemData.fCont = @(t,x1,x2) zeros(size(x1));
problemData.cDCont = @(t,x1,x2) zeros(size(x1));
problemData.gNCont = @(t,x1,x2) zeros(size(x1));
slot = @(x1, x2) double((x1 - 0.5).^2 + (x2 - 0.75).^2 <= 0.0225 & (x1 <= 0.475 | x1 >= 0.525 | x2 >= 0.85));
switch problemData.testcase
  case 'gauss_slot'   % Gaussian hump + slotted cylinder in the rotating field
    problemData = setdefault(problemData, 'jitter', 0);
    problemData.c0Cont = @(x1, x2) exp(-((x1 - 0.25).^2 + (x2 - 0.5).^2) / 0.01) + slot(x1, x2);
    problemData.u1Cont = @(t,x1,x2) 0.5 - x2;
    problemData.u2Cont = @(t,x1,x2) x1 - 0.5;
  case 'ensemble'     % one seeded instance: 8-mode streamfunction velocity, Gaussian hump
    problemData = setdefault(problemData, 'jitter', 0.2);
    prm = problemData.ensembleParams;
    [problemData.u1Cont, problemData.u2Cont] = streamfunctionVelocity(prm.k, prm.l, prm.a);
    problemData.c0Cont = @(x1, x2) exp(-((x1 - prm.centre(1)).^2 + (x2 - prm.centre(2)).^2) / prm.width^2);
  case 'adjoint'      % the gradient workload: 16 streamfunction modes with coefficients theta
    problemData = setdefault(problemData, 'jitter', 0);
    [k, l] = meshgrid(1:4, 1:4);
    problemData.modeK = reshape(k, 1, []);  problemData.modeL = reshape(l, 1, []);
    assert(isfield(problemData, 'theta') && numel(problemData.theta) == 16, ...
           'The adjoint case needs the 16 streamfunction coefficients theta.')
    [problemData.u1Cont, problemData.u2Cont] = streamfunctionVelocity(problemData.modeK, problemData.modeL, problemData.theta);
    problemData.c0Cont = @(x1, x2) exp(-((x1 - 0.4).^2 + (x2 - 0.45).^2) / 0.01);
end % switch
problemData = setdefault(problemData, 'meshSeed', 0);
jitter = problemData.jitter;  meshSeed = problemData.meshSeed;
problemData.generateGridData = @(hmax) domainSquareJittered(hmax, jitter, meshSeed);
problemData.generateMarkE0Tint = @(g) g.idE0T == 0;
problemData.generateMarkE0TbdrN = @(g) false(g.numT, 3);
problemData.generateMarkE0TbdrD = @(g) ~(g.markE0Tint | g.markE0TbdrN);
end % function

% Parameters of an ensemble instance drawn from problemData.instanceSeed: mesh level in {5,6,7},
% p in {1,2}, 8 modes (k, l in 1..3, a ~ N(0, 0.1^2)), hump centre in [0.2,0.8]^2, width in
% [0.05,0.15], mesh seed.  Matlab's generator is not numpy's, so the same seed gives another
% instance than the Python mirror; pass problemData.ensembleParams to run a given instance.
function prm = ensembleParams(problemData)
s = RandStream('mt19937ar', 'Seed', problemData.instanceSeed);
levels = [5 6 7];
prm.level = levels(randi(s, 3));
prm.p = randi(s, 2);
prm.k = randi(s, 3, 1, 8);  prm.l = randi(s, 3, 1, 8);
prm.a = 0.1 * randn(s, 1, 8);
prm.centre = 0.2 + 0.6 * rand(s, 1, 2);
prm.width = 0.05 + 0.1 * rand(s);
prm.meshSeed = randi(s, 2^31 - 1);
end % function

% u = (d psi/dy, -d psi/dx) of psi = sum_m a_m sin(k_m pi x) sin(l_m pi y): divergence-free and
% tangential to the unit square's boundary.
function [u1, u2] = streamfunctionVelocity(k, l, a)
u1 = @(t, x1, x2) sumModes(@(km, lm, am) am * (lm*pi) * sin(km*pi*x1) .* cos(lm*pi*x2), k, l, a, x1);
u2 = @(t, x1, x2) sumModes(@(km, lm, am) -am * (km*pi) * cos(km*pi*x1) .* sin(lm*pi*x2), k, l, a, x1);
end % function

function out = sumModes(term, k, l, a, x1)
out = zeros(size(x1));
for m = 1 : numel(a)
  out = out + term(k(m), l(m), a(m));
end % for
end % function
